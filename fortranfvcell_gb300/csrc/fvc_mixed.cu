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
// (default 0.1).
// Both stop on ||b - A x||2 <= refine_tol * ||b||2 recomputed in FP64.  Dot
// products and norms: each thread sums its rows with compensated FP32
// (TwoSum), the per-thread pairs are combined in FP64.  GB300 executes FP64
// at ~1/64 of its FP32 rate, so the iteration keeps the FP64 pipe idle.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "fvc_device.cuh"
#include "fvc_internal.h"
#include "fvc_tma.cuh"

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

// (s, c) += (s2, c2) for unevaluated FP32 pairs: TwoSum of the leading
// parts, the trailing parts added to the error, Fast2Sum renormalisation.
__device__ __forceinline__ void ff_add(float &s, float &c, float s2, float c2) {
  const float t = __fadd_rn(s, s2);
  const float bp = __fsub_rn(t, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(s2, bp));
  const float cc = __fadd_rn(__fadd_rn(c, c2), err);
  s = __fadd_rn(t, cc);
  c = __fsub_rn(cc, __fsub_rn(s, t));
}

// Grid-wide deterministic sum of NV compensated FP32 partials per thread.
// Warps reduce their pairs with an FP32 butterfly (FP32 pair arithmetic,
// not FP64: GB300 runs FP64 at ~2 lanes per clock per SM, and a block of
// 1024 threads each doing FP64 shuffles and divisions costs microseconds
// per reduction); warp 0 combines the warps, converts the block's pair to
// FP64 once, publishes it and arrives on the grid counter (release), waits
// for every block's arrival (acquire) and sums all partials in block order
// itself, so every block holds identical totals after two trips to L2.
// Lane 0 of warp 0 then calls f(totals) -- the place for the iteration's scalar FP64
// work, which it publishes through shared memory -- and one __syncthreads
// hands the results to the block.  Returns false when a wait exceeded its
// bound (gs.err set).
template <int NV, typename F>
__device__ __forceinline__ bool grid_allreduce_ff(const GridSync &gs, unsigned int &episode,
                                                  const CSum (&v)[NV], float2 *red2, F &&f) {
  __shared__ int s_ok;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    float s = v[q].s, c = v[q].c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
      const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
      ff_add(s, c, s2, c2);
    }
    if (lane == 0) red2[q * 32 + warp] = make_float2(s, c);
  }
  if (threadIdx.x == 0) s_ok = 1;
  __syncthreads();
  const unsigned int ep = ++episode;
  if (gs.cluster) {  // one thread-block cluster: cluster_exchange
    __shared__ double s_slot[2][kMaxNV];
    if (warp == 0) {
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const float2 w = (lane < nwarps) ? red2[q * 32 + lane] : make_float2(0.0f, 0.0f);
        float s = w.x, c = w.y;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
          const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
          ff_add(s, c, s2, c2);
        }
        if (lane == 0) s_slot[ep & 1u][q] = (double)s + (double)c;
      }
    }
    double t[NV];
    cluster_exchange<NV>(s_slot, ep, t);
    if (threadIdx.x == 0) f(t);
    __syncthreads();
    return true;
  }
  if (warp == 0) {
    const unsigned int nb = gs.nblocks;
    double *part = gs.partials + (size_t)(ep & 3u) * kMaxNV * nb;
    double bsum[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const float2 w = (lane < nwarps) ? red2[q * 32 + lane] : make_float2(0.0f, 0.0f);
      float s = w.x, c = w.y;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
        const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
        ff_add(s, c, s2, c2);
      }
      bsum[q] = (double)s + (double)c;
    }
    bool ok = true;
    double t[NV];
    if (nb == 1) {  // one block: its sum is the total (same value)
#pragma unroll
      for (int q = 0; q < NV; ++q) t[q] = bsum[q];
    } else {
      // publish the block's partials, then wait until every block has
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) part[(size_t)q * nb + (blockIdx.x - gs.base)] = bsum[q];
        red_add_release(gs.count, 1u);
        const unsigned int target = ep * nb;
        const uint64_t t0 = global_ns();
        unsigned int spins = 0;
        while (ld_acquire(gs.count) < target) {
          if (*(volatile int *)gs.err != 0) {
            ok = false;
            break;
          }
          if ((++spins & 255u) == 0 && global_ns() - t0 > kBarrierTimeoutNs) {
            atomicExch(gs.err, 7 /* FVC_ERR_TIMEOUT */);
            ok = false;
            break;
          }
          __nanosleep(20);
        }
      }
      ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      // every block sums the partials itself, in block order (identical
      // totals everywhere; no second round trip through a release flag)
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        double u = 0.0;
        if (ok) {
          const double *pp = part + (size_t)q * nb;
          for (unsigned int b = lane; b < nb; b += 32) u = __dadd_rn(u, __ldcg(pp + b));
        }
        t[q] = warp_sum(u);
      }
    }
    if (lane == 0) {
      if (ok)
        f(t);
      else
        s_ok = 0;
    }
  }
  __syncthreads();
  return s_ok != 0;
}

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

// Layout scan: flags[0] = 1 if some column offset (col - row) of a slot
// with a nonzero value needs more than 16 bits, flags[1] / flags[2] =
// smallest / largest slice width.  Slots holding 0 (the reference's ELLPACK
// padding: column 1, value 0, src/EllPack.f:19-42) add exactly 0 in the
// difference form whatever column they name, so the FP32 operator points
// them at their own row (offset 0) and they do not count here.
__global__ void scan_slices(int n, int nslices, const int64_t *__restrict__ sptr,
                            const int *__restrict__ col, const double *__restrict__ val,
                            int *__restrict__ flags) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += nw) {
    const int row = s * 32 + lane;
    const int64_t base = sptr[s];
    const int wd = (int)((sptr[s + 1] - base) >> 5);
    bool wide = false;
    for (int k = 0; k < wd; ++k) {
      const int64_t q = base + 32 * k + lane;
      const int d = (row < n && val[q] != 0.0) ? col[q] - row : 0;
      if (d < -32768 || d > 32767) wide = true;
    }
    if (__any_sync(0xffffffffu, wide) && lane == 0) atomicExch(flags, 1);
    if (lane == 0) {
      atomicMin(flags + 1, wd);
      atomicMax(flags + 2, wd);
    }
  }
}

// Slot of (lane, k) in a slice of the FP32 operator that starts at slot
// dbase.  Width-4 uniform layout (ell_w == 4): row-major inside the slice,
// a row's four slots contiguous (4 lane + k), so a lane reads its row's
// weights with one 16-byte load and its offsets with one 8-byte load.
// Otherwise column-major as in SELL-32 (32 k + lane): a warp's k-th slots
// are one coalesced 128-byte line.
__host__ __device__ __forceinline__ int64_t f32_slot(int64_t dbase, int ell_w, int lane, int k) {
  return (ell_w == 4) ? dbase + 4 * lane + k : dbase + 32 * k + lane;
}

// e_i (FP64 sum, rounded once), Jacobi 1/m, the FP32 weights, the 16-bit
// column offsets (col - row) and the per-slice "has excess" flags.  With
// ell_w > 0 the weights and offsets are laid out with every slice ell_w
// slots wide (slice s at slot 32 ell_w s); the slots a narrower slice lacks
// get weight 0 and offset 0, which add exactly 0 to every row sum.
// check16: the kernels read col16, so a nonzero slot whose offset does not
// fit 16 bits (possible only where the layout scan saw a 0 there) sets *bad.
__global__ void build_f32_operator(int n, int nslices, const int64_t *__restrict__ sptr,
                                   const int *__restrict__ col, const double *__restrict__ val,
                                   const double *__restrict__ jac, float *__restrict__ w32,
                                   float *__restrict__ e32, float *__restrict__ minv32,
                                   int16_t *__restrict__ col16, uint8_t *__restrict__ sflag,
                                   int ell_w, int check16, int *__restrict__ bad) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += nw) {
    const int row = s * 32 + lane;
    const int64_t base = sptr[s];
    const int wd = (int)((sptr[s + 1] - base) >> 5);
    const int64_t dbase = (ell_w > 0) ? (int64_t)s * 32 * ell_w : base;
    double off = 0.0;  // sum of a_ik over true off-diagonal slots
    for (int k = 0; k < wd; ++k) {
      const int64_t q = base + 32 * k + lane;
      const bool diag_slot = (row < n) && (col[q] == row);
      const double a = (row < n && !diag_slot) ? val[q] : 0.0;
      off += a;
      const int64_t o = f32_slot(dbase, ell_w, lane, k);
      const int d = (row < n && a != 0.0) ? col[q] - row : 0;
      if (check16 && (d < -32768 || d > 32767)) atomicExch(bad, 1);
      w32[o] = (a != 0.0) ? (float)(-a) : 0.0f;
      col16[o] = (int16_t)d;
    }
    for (int k = wd; k < ell_w; ++k) {
      const int64_t o = f32_slot(dbase, ell_w, lane, k);
      w32[o] = 0.0f;
      col16[o] = 0;
    }
    float ev = 0.0f;
    if (row < n) {
      const double m = jac[row];
      double e = m + off;
      e = fmin(fmax(e, -kF32Clamp), kF32Clamp);
      ev = (float)e;
      e32[row] = ev;
      minv32[row] = (fabs(m) > 1.0e37 || m == 0.0) ? 0.0f : (float)(1.0 / m);
    }
    const bool any_e = __any_sync(0xffffffffu, ev != 0.0f);
    if (lane == 0) sflag[s] = any_e ? 1 : 0;
  }
}

struct MArgs {
  SellView<double> A;   // FP64 matrix (true residuals)
  const float *w32;     // weights per slot
  const float *e32;     // row excess
  const float *minv;    // Jacobi 1/m (0 on rows whose m is beyond FP32)
  const int16_t *col16; // column offsets (col - row), when col16_ok
  int ell_w;            // > 0: w32/col16 hold every slice ell_w slots wide
  const uint8_t *sflag; // per slice: some row has e_i != 0
  const int *f32_bad;   // nonzero: the 16-bit offsets no longer describe A
  const double *jac;    // m in FP64
  const double *b;
  double *x;
  float *rs, *pa, *pb, *q, *r0, *v, *t, *z;
  float *rsl;           // CG: low part of the residual (FP32 pair rs + rsl)
  float *pal, *pbl;     // CG: low parts of the search directions in pa, pb
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
  double *trace;        // (iteration, relres) per residual replacement (may be null)
  float *history;       // recursive relres per iteration (may be null)
  // one system of a batch: its slices [grp_s0, grp_s1) over grp_nb blocks
  // from block grp_base (grp_nb = 0: the whole matrix over the grid)
  int grp_s0 = 0, grp_s1 = 0, grp_nb = 0, grp_base = 0;
};

// the block that writes the system's results
__device__ __forceinline__ bool mlead(const MArgs &a) {
  return blockIdx.x == (a.grp_nb > 0 ? (unsigned)a.grp_base : 0u);
}

// (A y)_row in FP32 difference form, y supplied by a functor.
template <typename YF>
__device__ __forceinline__ float arow32(const MArgs &a, int s, int lane, int row, YF yf) {
  if (a.ell_w == 4) {  // width 4, row-major in the slice: one 16-B and one 8-B load
    const int64_t base = (int64_t)s * 128 + 4 * lane;
    const float4 w = ld_stream4(a.w32 + base);
    const uint2 c = ld_stream_u2(a.col16 + base);
    const float yi = yf(row);
    float t = ld_stream(a.e32 + row) * yi;
    int k4[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      k4[k] = row + off16(c, k);
      FVC_CHK((unsigned)k4[k] < (unsigned)a.A.n, a.A.chk, kChkOffset, k4[k] = row);
    }
    t = fmaf(w.x, yi - yf(k4[0]), t);
    t = fmaf(w.y, yi - yf(k4[1]), t);
    t = fmaf(w.z, yi - yf(k4[2]), t);
    t = fmaf(w.w, yi - yf(k4[3]), t);
    return t;
  }
  if (a.ell_w == 3) {  // width 3, column-major: the loads issued before the gathers
    const int64_t base = (int64_t)s * 96 + lane;
    float w[3];
    int c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      w[k] = ld_stream(a.w32 + base + 32 * k);
      c[k] = row + (int)ld_stream16(a.col16 + base + 32 * k);
      FVC_CHK((unsigned)c[k] < (unsigned)a.A.n, a.A.chk, kChkOffset, c[k] = row);
    }
    const float yi = yf(row);
    float t = ld_stream(a.e32 + row) * yi;
#pragma unroll
    for (int k = 0; k < 3; ++k) t = fmaf(w[k], yi - yf(c[k]), t);
    return t;
  }
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
      FVC_CHK((unsigned)c[k] < (unsigned)a.A.n, a.A.chk, kChkColumn, c[k] = row);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < w) t = fmaf(v[k], yi - yf(c[k]), t);
    return t;
  }
  for (int k = 0; k < w; ++k) {
    int c = ld_stream(cp + 32 * k);
    FVC_CHK((unsigned)c < (unsigned)a.A.n, a.A.chk, kChkColumn, c = row);
    t = fmaf(ld_stream(vp + 32 * k), yi - yf(c), t);
  }
  return t;
}

struct MPart {
  int lane, warp, nwarps, sb, se, n;
  // this block's slices: of the whole matrix over the grid, or of the
  // batch system a belongs to over that system's blocks
  __device__ explicit MPart(const MArgs &a) {
    lane = threadIdx.x & 31;
    warp = threadIdx.x >> 5;
    nwarps = blockDim.x >> 5;
    const int s0 = a.grp_nb > 0 ? a.grp_s0 : 0;
    const int s1 = a.grp_nb > 0 ? a.grp_s1 : a.A.nslices;
    const int nb = a.grp_nb > 0 ? a.grp_nb : (int)gridDim.x;
    const int rank = (int)blockIdx.x - (a.grp_nb > 0 ? a.grp_base : 0);
    const int spb = (s1 - s0 + nb - 1) / nb;
    sb = s0 + rank * spb;
    se = min(s1, sb + spb);
    n = a.A.n;
  }
};

#define MFOR_ROWS(P)                                               \
  for (int s_ = (P).sb + (P).warp; s_ < (P).se; s_ += (P).nwarps) \
    for (int row = s_ * 32 + (P).lane, once_ = 1; once_ && row < (P).n; once_ = 0)

// The same rows two slices per warp step: f(s, row, ok) gets this step's
// two slices (s, s + nwarps), so a body that loads both rows' operands
// before it stores either result keeps two rows' gathers in flight (the
// warp's loads of one row otherwise wait on the stores of the one before,
// which the compiler cannot move past them).  A missing second slice, or a
// second row at or beyond n, comes as a copy of the first (the same slice,
// lane and row, so every load it makes is the first row's own, in bounds)
// with ok = false: its results are dropped.  A lane whose first row is at
// or beyond n (the last slice's padding) has nothing left to do.  The rows
// are visited in the order of MFOR_ROWS, so sums over them are the same.
template <typename F>
__device__ __forceinline__ void mfor_rows2(const MPart &P, F &&f) {
  for (int s = P.sb + P.warp; s < P.se; s += 2 * P.nwarps) {
    const int ra = s * 32 + P.lane;
    if (ra >= P.n) break;  // later slices of this warp are further on
    const int s1 = s + P.nwarps;
    const int rb = s1 * 32 + P.lane;
    const bool second = s1 < P.se && rb < P.n;
    const int sl[2] = {s, second ? s1 : s};
    const int rw[2] = {ra, second ? rb : ra};
    const bool ok[2] = {true, second};
    f(sl, rw, ok);
  }
}

// FP64 residual sweep: rs = b - A x rounded to FP32.  Returns ||b-Ax||^2,
// ||b||^2, rs.(rs/m) and ||b-Ax||^2 over the rows the FP32 iteration moves
// (FP64 sums).
__device__ __forceinline__ bool residual_sweep(const MArgs &a, unsigned int &ep, bool zero_x,
                                               double (&out)[4], double *red) {
  const MPart P(a);
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

// x += e (+ a deferred alpha*p) in FP64 and e = 0, own rows; a barrier
// must follow.  Rows whose
// diagonal is beyond FP32 range (1/m = 0: the pressure pin) are frozen in
// the FP32 iteration; they take one FP64 Jacobi step on their current
// residual estimate instead, which solves such a row to FP64 accuracy.
__device__ __forceinline__ void fold_correction(const MArgs &a, const float *ppend = nullptr,
                                                const float *ppend_lo = nullptr,
                                                double apend = 0.0) {
  const MPart P(a);
  MFOR_ROWS(P) {
    const float2 ev = a.e[row];
    double dx = (double)ev.x + (double)ev.y;
    if (ppend)  // a deferred alpha*p (p an FP32 pair)
      dx = fma(apend, (double)ppend[row] + (double)ppend_lo[row], dx);
    const double m = a.jac[row];
    if (a.minv[row] == 0.0f && m != 0.0) {
      // the frozen row's residual grows to the size of the neighbours' x
      // over a cycle; the Jacobi step needs all of it (both pair parts)
      const double rr = (double)a.rs[row] + (a.rsl ? (double)a.rsl[row] : 0.0);
      dx += rr / m;
    }
    a.x[row] = a.x[row] + dx;
    a.e[row] = make_float2(0.0f, 0.0f);
  }
}

// The search direction is carried as an unevaluated FP32 pair (hi, lo):
// rounding p = z + beta p_prev to one FP32 number each iteration perturbs
// the direction by eps32 relative and, on the Jacobi-scaled Neumann
// systems (lowest eigenvalues near eps32), sometimes stalls the last decade
// of convergence for hundreds of iterations; the pair removes that.  The
// operator is applied to p_hi (the FP32 value of p); the correction
// e += alpha p takes both parts.
struct Dir {
  const float *ph, *pl;  // p_prev (hi, lo)
  float *ch, *cl;        // p (hi, lo), written by phase A
};

// p = z + (bh + bl)(ph + pl) as an FP32 pair: the product's rounding error
// comes from an FMA, the sum uses TwoSum, then a Fast2Sum renormalisation.
__device__ __forceinline__ float2 p_update(float z, float bh, float bl, float ph, float pl) {
  const float th = __fmul_rn(bh, ph);
  const float terr = fmaf(bh, ph, -th);
  const float tl = fmaf(bh, pl, fmaf(bl, ph, terr));
  const float s = __fadd_rn(th, z);
  const float bp = __fsub_rn(s, th);
  const float err = __fadd_rn(__fsub_rn(th, __fsub_rn(s, bp)), __fsub_rn(z, bp));
  const float lo = __fadd_rn(tl, err);
  const float hi = __fadd_rn(s, lo);
  return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

// CG phase A with plain loads: p = z + beta p_prev (formed at each gathered
// neighbour), q = A p_hi, returns p_hi.q.  Two slices per warp step
// (mfor_rows2).
template <bool kFirst>
__device__ __forceinline__ CSum cg_phase_a(const MArgs &a, const MPart &P, float bh, float bl,
                                           const Dir &d) {
  CSum cpq;
  const float *__restrict__ z = a.z;
  auto pf = [&](int k) -> float2 {
    return kFirst ? make_float2(z[k], 0.0f) : p_update(z[k], bh, bl, d.ph[k], d.pl[k]);
  };
  mfor_rows2(P, [&](const int(&sl)[2], const int(&rw)[2], const bool(&ok)[2]) {
    float2 pi[2];
    float t[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      pi[u] = pf(rw[u]);
      t[u] = arow32(a, sl[u], P.lane, rw[u], [&](int k) { return pf(k).x; });
    }
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (ok[u]) {
        d.ch[rw[u]] = pi[u].x;
        d.cl[rw[u]] = pi[u].y;
        a.q[rw[u]] = t[u];
        if (kFirst) a.e[rw[u]] = make_float2(0.0f, 0.0f);
        cpq.add(pi[u].x * t[u]);
      }
  });
  return cpq;
}

// (hi, lo) += (ah + al)(ph + pl) for the correction (FP32 pairs).
__device__ __forceinline__ float2 df_axpy2(float2 e, float ah, float al, float ph, float pl) {
  const float th = __fmul_rn(ah, ph);
  const float terr = fmaf(ah, ph, -th);
  const float tl = fmaf(ah, pl, fmaf(al, ph, terr));
  const float s = __fadd_rn(e.x, th);
  const float bp = __fsub_rn(s, e.x);
  const float err = __fadd_rn(__fsub_rn(e.x, __fsub_rn(s, bp)), __fsub_rn(th, bp));
  const float lo = __fadd_rn(__fadd_rn(e.y, tl), err);
  const float hi = __fadd_rn(s, lo);
  return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

// One row of CG phase B: e += a1 p_prev + alpha p (kUpdE), r -= alpha q
// (an FP32 pair with kPair), z = r/m; accumulates r.z and r.r (moving rows).
template <bool kPair, bool kUpdE>
__device__ __forceinline__ void cg_row_b(float a1, float a1_lo, float alpha, float alpha_lo,
                                         float qv, float rv, float rl, float mv, float2 ev,
                                         float p1h, float p1l, float pvh, float pvl, float2 &eo,
                                         float &ro, float &rlo, float &zo, CSum &crz, CSum &crr) {
  if (kUpdE) eo = df_axpy2(df_axpy2(ev, a1, a1_lo, p1h, p1l), alpha, alpha_lo, pvh, pvl);
  float r;
  if (kPair) {
    const float2 rp = df_axpy(make_float2(rv, rl), -alpha, -alpha_lo, qv);
    r = rp.x;
    rlo = rp.y;
  } else {
    r = fmaf(-alpha, qv, rv);
  }
  const float zz = r * mv;
  ro = r;
  zo = zz;
  crz.add(r * zz);
  if (mv != 0.0f) crr.add(r * r);
}

// CG phase B with plain loads.
template <bool kPair, bool kUpdE>
__device__ __forceinline__ void cg_phase_b(const MArgs &a, const MPart &P, float a1, float a1_lo,
                                           float alpha, float alpha_lo, const Dir &d, CSum &crz,
                                           CSum &crr) {
  mfor_rows2(P, [&](const int(&sl)[2], const int(&rw)[2], const bool(&ok)[2]) {
    float qv[2], rv[2], rl[2], mv[2], p1h[2], p1l[2], pvh[2], pvl[2];
    float2 ev[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int row = rw[u];
      qv[u] = a.q[row];
      rv[u] = a.rs[row];
      rl[u] = kPair ? a.rsl[row] : 0.0f;
      mv[u] = a.minv[row];
      ev[u] = kUpdE ? a.e[row] : make_float2(0.0f, 0.0f);
      p1h[u] = kUpdE ? d.ph[row] : 0.0f;
      p1l[u] = kUpdE ? d.pl[row] : 0.0f;
      pvh[u] = kUpdE ? d.ch[row] : 0.0f;
      pvl[u] = kUpdE ? d.cl[row] : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (ok[u]) {
        const int row = rw[u];
        float2 eo;
        float ro, rlo = 0.0f, zo;
        cg_row_b<kPair, kUpdE>(a1, a1_lo, alpha, alpha_lo, qv[u], rv[u], rl[u], mv[u], ev[u],
                               p1h[u], p1l[u], pvh[u], pvl[u], eo, ro, rlo, zo, crz, crr);
        if (kUpdE) a.e[row] = eo;
        a.rs[row] = ro;
        if (kPair) a.rsl[row] = rlo;
        a.z[row] = zo;
      }
  });
}

// ---------------------------------------------------------------------
// Staged phases.  Each block walks its slice range in chunks of 32 slices
// (1024 rows: one slice per warp in phase A, one row per thread in phase
// B).  Warp 0 keeps bulk copies (TMA) running ahead into shared memory,
// so the streams arrive without occupying registers or warps.
//  * Phase A: z and p_prev (both parts) of each chunk of the window land
//    kLandAhead chunks ahead; one pass per row then forms the p pair once,
//    writes p_hi into a ring of kPRingRows rows of shared memory (indexed
//    by (row - first row of the block) mod kPRingRows) and the own rows'
//    pair to global memory.  The ring holds chunks i-3 .. i+4 while chunk i
//    is computed, so q = A p gathers every neighbour within +-3072 rows
//    from shared memory (under the RCM numbering of a 2-D mesh with up to
//    ~3000 rows per level, all of them); one further away is formed from
//    global memory.  The chunk's weights and column offsets come through
//    kAStages stages.  The window reaches into the neighbouring blocks'
//    rows; the first window chunks (i-3 .. i+3 of chunk 0) are formed with
//    plain loads.
//  * Phase B stages all of its row vectors in kBStages stages.
// The two phases reuse the same shared memory (a grid barrier separates
// them).  A chunk with more than kStSlotCap slots (mean row width above 5)
// reads its weights and offsets from global memory instead.
constexpr int kStChunkSlices = 32;
constexpr int kStagedRows = 524288;              // staged CG from this many rows
constexpr int kStRows = kStChunkSlices * kSlice;  // = threads per block
constexpr int kStSlotCap = kStRows * 5;
constexpr int kWinHalo = 3;                      // gathers from chunks i-3 .. i+3
constexpr int kWinSpan = (2 * kWinHalo + 1) * kStRows;
constexpr int kPRingRows = 8 * kStRows;          // chunks i-3 .. i+4
constexpr int kLandSlots = 4;
constexpr int kLandAhead = 3;                    // landing copies in flight
constexpr int kAStages = 4;
constexpr int kBStages = 5;
// phase A: p ring | landing slots (z | pp_hi | pp_lo) | stages (w32 | col16)
constexpr uint32_t kLandBytes = 3 * kStRows * 4;
constexpr uint32_t kL_Base = kPRingRows * 4;
constexpr uint32_t kA_Base = kL_Base + kLandSlots * kLandBytes;
constexpr uint32_t kA_C = kStSlotCap * 4;
constexpr uint32_t kA_Bytes = kA_C + kStSlotCap * 2;
// phase B stage: q | rs | rsl | minv | p1h | p1l | pvh | pvl (1024 floats each) | e[1024] float2
constexpr uint32_t kB_Q = 0, kB_RS = 1 * kStRows * 4, kB_RSL = 2 * kStRows * 4,
                   kB_MINV = 3 * kStRows * 4, kB_P1H = 4 * kStRows * 4,
                   kB_P1L = 5 * kStRows * 4, kB_PVH = 6 * kStRows * 4,
                   kB_PVL = 7 * kStRows * 4, kB_E = 8 * kStRows * 4;
constexpr uint32_t kB_Bytes = kB_E + kStRows * 8;
constexpr uint32_t kRegionA = kA_Base + kAStages * kA_Bytes;
constexpr uint32_t kRegionB = kBStages * kB_Bytes;
constexpr uint32_t kStHeader = 256;
constexpr size_t kStSmem = kStHeader + (kRegionA > kRegionB ? kRegionA : kRegionB);
static_assert(kA_Bytes % 128 == 0 && kB_Bytes % 128 == 0 && kA_Base % 128 == 0, "alignment");
static_assert(kStSmem + 3072 <= 227 * 1024, "shared memory per block");
static_assert(kLandAhead + 1 == kLandSlots, "landing ring");

struct StHdr {
  uint64_t land[kLandSlots];  // landing slot filled
  uint64_t sa[kAStages];      // phase-A stage filled
  uint64_t sb[kBStages];      // phase-B stage filled
  int64_t base[kAStages];     // first slot of the chunk in each phase-A stage
  int ok[kAStages];           // 1: its weights and offsets are staged
};
static_assert(sizeof(StHdr) <= kStHeader, "stage header");

// Running counts of the copies issued into each ring (the same in every
// thread): ring slot = count % size, mbarrier parity = (count / size) & 1.
struct StCount {
  uint32_t land = 0, sa = 0, sb = 0;
};

__device__ __forceinline__ unsigned char *st_region(unsigned char *smem) {
  return smem + kStHeader;
}

// Chunk boundaries sptr[min(se, sb + 32 j)], cached 32 at a time in the
// lanes of warp 0 (every lane calls with the same j).
struct Bounds {
  int64_t v;
  int jb;
};
__device__ __forceinline__ int64_t bounds_get(Bounds &B, const MArgs &a, const MPart &P, int j) {
  if (j < B.jb || j >= B.jb + 32) {
    B.jb = j;
    const int s = min(P.se, P.sb + kStChunkSlices * (j + P.lane));
    B.v = a.A.sptr[s];
  }
  return __shfl_sync(0xffffffffu, B.v, j - B.jb);
}

__device__ __forceinline__ int st_chunks(const MPart &P) {
  return (P.se > P.sb) ? (P.se - P.sb + kStChunkSlices - 1) / kStChunkSlices : 0;
}

// Lane 0 of warp 0: z and p_prev (hi, lo) of window chunk j (rows R0 +
// 1024 j .., j >= 1, clipped to the padded row range) into landing slot seq.
template <bool kFirst>
__device__ __forceinline__ void issue_land(const MArgs &a, const MPart &P, unsigned char *smem,
                                           uint32_t seq, int j, int nrows, const Dir &d) {
  StHdr *H = reinterpret_cast<StHdr *>(smem);
  const uint32_t slot = seq % kLandSlots;
  const int c0 = P.sb * kSlice + j * kStRows;
  const int hi = min(c0 + kStRows, nrows);
  uint64_t *bar = &H->land[slot];
  if (hi <= c0) {
    mbar_arrive_expect_tx(bar, 0);
    return;
  }
  const uint32_t bytes = (uint32_t)(hi - c0) * 4u;
  unsigned char *dst = st_region(smem) + kL_Base + slot * kLandBytes;
  mbar_arrive_expect_tx(bar, kFirst ? bytes : 3u * bytes);
  bulk_g2s(dst, a.z + c0, bytes, bar);
  if (!kFirst) {
    bulk_g2s(dst + kStRows * 4, d.ph + c0, bytes, bar);
    bulk_g2s(dst + 2 * kStRows * 4, d.pl + c0, bytes, bar);
  }
}

// Warp 0: weights and column offsets of chunk j into phase-A stage seq.
__device__ __forceinline__ void issue_slots(const MArgs &a, const MPart &P, unsigned char *smem,
                                            Bounds &B, uint32_t seq, int j) {
  StHdr *H = reinterpret_cast<StHdr *>(smem);
  const int64_t s0 = bounds_get(B, a, P, j);
  const int64_t s1 = bounds_get(B, a, P, j + 1);
  if (P.lane != 0) return;
  const uint32_t stg = seq % kAStages;
  const int64_t nsl = s1 - s0;
  const bool ok = nsl <= kStSlotCap;
  H->base[stg] = s0;
  H->ok[stg] = ok ? 1 : 0;
  uint64_t *bar = &H->sa[stg];
  unsigned char *b = st_region(smem) + kA_Base + stg * kA_Bytes;
  mbar_arrive_expect_tx(bar, (ok && nsl > 0) ? (uint32_t)nsl * 6u : 0u);
  if (ok && nsl > 0) {
    bulk_g2s(b, a.w32 + s0, (uint32_t)nsl * 4u, bar);
    bulk_g2s(b + kA_C, a.col16 + s0, (uint32_t)nsl * 2u, bar);
  }
}

// Lane 0 of warp 0: chunk j of a uniform-width-kW layout (slice s starts
// at slot 32 kW s) into phase-A stage seq.
template <int kW>
__device__ __forceinline__ void issue_slots_u(const MArgs &a, const MPart &P, unsigned char *smem,
                                              uint32_t seq, int j) {
  StHdr *H = reinterpret_cast<StHdr *>(smem);
  const uint32_t stg = seq % kAStages;
  const int c0 = P.sb + kStChunkSlices * j;
  const int c1 = min(P.se, c0 + kStChunkSlices);
  const int64_t s0 = (int64_t)c0 * kSlice * kW;
  const uint32_t nsl = (uint32_t)(c1 - c0) * kSlice * kW;
  uint64_t *bar = &H->sa[stg];
  unsigned char *b = st_region(smem) + kA_Base + stg * kA_Bytes;
  mbar_arrive_expect_tx(bar, nsl * 6u);
  bulk_g2s(b, a.w32 + s0, nsl * 4u, bar);
  bulk_g2s(b + kA_C, a.col16 + s0, nsl * 2u, bar);
}

// Forms the p pair of row r (from z and p_prev given), puts p_hi in the
// ring and stores the pair when the row is the block's own.
template <bool kFirst>
__device__ __forceinline__ void p_form(float *ring, int r, int R0, int Rend, int n, float zr,
                                       float bh, float bl, float phr, float plr, const Dir &d) {
  const float2 p = kFirst ? make_float2(zr, 0.0f) : p_update(zr, bh, bl, phr, plr);
  ring[(r - R0) & (kPRingRows - 1)] = p.x;
  if (r >= R0 && r < Rend && r < n) {
    d.ch[r] = p.x;
    d.cl[r] = p.y;
  }
}

// Lane 0 of warp 0: the first phase-A stages of a uniform-width layout.
// They copy matrix weights and offsets only (constants), so they may be
// issued before the grid reduction that ends phase B; the next phase A
// then finds them in flight (pre = true).
template <int kW>
__device__ __forceinline__ void prefetch_a(const MArgs &a, const MPart &P, unsigned char *smem,
                                           const StCount &cnt) {
  if (P.warp == 0 && P.lane == 0) {
    fence_proxy_async_smem();
    const int nch = st_chunks(P);
    for (int j = 0; j < kAStages - 1 && j < nch; ++j)
      issue_slots_u<kW>(a, P, smem, cnt.sa + (uint32_t)j, j);
  }
}

// The prefetched phase-A stages complete before the block leaves the loop
// without a phase A to consume them (stop, maxit, a reduction that gave up).
__device__ __forceinline__ void drain_prefetch_a(const MPart &P, unsigned char *smem,
                                                 const StCount &cnt) {
  StHdr *H = reinterpret_cast<StHdr *>(smem);
  const int nch = st_chunks(P);
  for (int j = 0; j < kAStages - 1 && j < nch; ++j) {
    const uint32_t seq = cnt.sa + (uint32_t)j;
    mbar_drain(&H->sa[seq % kAStages], (seq / kAStages) & 1u);
  }
}

// Staged phase A: p = z + beta p_prev, q = A p_hi, returns p_hi.q.  Same
// arithmetic, in the same order, as cg_phase_a.  kW > 0: every slice has
// width kW (slot offsets follow from the slice index; no slice-pointer
// loads, no capacity check, fixed unrolled row loop); kW == 0: general.
template <bool kFirst, int kW>
__device__ __forceinline__ CSum cg_phase_a_st(const MArgs &a, const MPart &P, float bh, float bl,
                                              const Dir &d, unsigned char *smem, StCount &cnt,
                                              bool pre = false) {
  StHdr *H = reinterpret_cast<StHdr *>(smem);
  CSum cpq;
  const int nch = st_chunks(P);
  if (nch == 0) return cpq;
  const int nrows = a.A.nslices * kSlice;
  const int R0 = P.sb * kSlice, Rend = P.se * kSlice;
  const int jlast = nch - 1 + kWinHalo;  // last window chunk any row needs
  float *ring = reinterpret_cast<float *>(st_region(smem));
  Bounds B;
  B.jb = -64;
  B.v = 0;
  if (P.warp == 0) {
    if (P.lane == 0) {
      fence_proxy_async_global();
      fence_proxy_async_smem();
      for (int j = kWinHalo + 1; j <= jlast && j <= kWinHalo + kLandAhead; ++j)
        issue_land<kFirst>(a, P, smem, cnt.land + (j - kWinHalo - 1), j, nrows, d);
    }
    for (int j = 0; j < kAStages - 1 && j < nch && !(kW > 0 && pre); ++j) {
      if (kW > 0) {
        if (P.lane == 0) issue_slots_u<kW>(a, P, smem, cnt.sa + j, j);
      } else {
        issue_slots(a, P, smem, B, cnt.sa + j, j);
      }
    }
  }
  // window chunks -3 .. 3 with plain loads (one row of each per thread)
  {
    float zr[2 * kWinHalo + 1], phr[2 * kWinHalo + 1], plr[2 * kWinHalo + 1];
#pragma unroll
    for (int jj = 0; jj < 2 * kWinHalo + 1; ++jj) {
      const int j = jj - kWinHalo, r = R0 + j * kStRows + (int)threadIdx.x;
      const bool in = j <= jlast && r >= 0 && r < nrows;
      zr[jj] = in ? a.z[r] : 0.0f;
      phr[jj] = (in && !kFirst) ? d.ph[r] : 0.0f;
      plr[jj] = (in && !kFirst) ? d.pl[r] : 0.0f;
    }
#pragma unroll
    for (int jj = 0; jj < 2 * kWinHalo + 1; ++jj) {
      const int j = jj - kWinHalo, r = R0 + j * kStRows + (int)threadIdx.x;
      if (j <= jlast && r >= 0 && r < nrows)
        p_form<kFirst>(ring, r, R0, Rend, P.n, zr[jj], bh, bl, phr[jj], plr[jj], d);
    }
  }
  // this warp's slice bounds and its rows' excess e_i, one chunk ahead
  int64_t my0 = 0, my1 = 0;
  float myex = 0.0f;
  {
    const int s = P.sb + P.warp;
    if (s < P.se) {
      if (kW == 0) {
        my0 = a.A.sptr[s];
        my1 = a.A.sptr[s + 1];
      }
      if (a.sflag[s] && s * kSlice + P.lane < P.n) myex = ld_stream(a.e32 + s * kSlice + P.lane);
    }
  }
  __syncthreads();
  for (int i = 0; i < nch; ++i) {
    if (P.warp == 0) {
      const int jl = i + kWinHalo + 1 + kLandAhead;
      if (P.lane == 0 && jl <= jlast)
        issue_land<kFirst>(a, P, smem, cnt.land + (jl - kWinHalo - 1), jl, nrows, d);
      if (i + kAStages - 1 < nch) {
        if (kW > 0) {
          if (P.lane == 0) issue_slots_u<kW>(a, P, smem, cnt.sa + i + kAStages - 1, i + kAStages - 1);
        } else {
          issue_slots(a, P, smem, B, cnt.sa + i + kAStages - 1, i + kAStages - 1);
        }
      }
    }
    const int s = P.sb + kStChunkSlices * i + P.warp;
    // next chunk's slice bounds, loaded while this chunk is processed
    int64_t n0 = 0, n1 = 0;
    float nex = 0.0f;
    if (s + kStChunkSlices < P.se) {
      const int sn = s + kStChunkSlices, rn = sn * kSlice + P.lane;
      if (kW == 0) {
        n0 = a.A.sptr[sn];
        n1 = a.A.sptr[sn + 1];
      }
      if (a.sflag[sn] && rn < P.n) nex = ld_stream(a.e32 + rn);
    }
    // form p for window chunk i+4 (used from the next chunk on)
    const int jf = i + kWinHalo + 1;
    if (jf <= jlast) {
      const uint32_t sq = cnt.land + (uint32_t)i;
      const uint32_t slot = sq % kLandSlots;
      mbar_wait(&H->land[slot], (sq / kLandSlots) & 1u, a.gs.err);
      const int r = R0 + jf * kStRows + (int)threadIdx.x;
      if (r < nrows) {
        const float *L = reinterpret_cast<const float *>(st_region(smem) + kL_Base +
                                                         slot * kLandBytes);
        const int t = threadIdx.x;
        p_form<kFirst>(ring, r, R0, Rend, P.n, L[t], bh, bl, kFirst ? 0.0f : L[kStRows + t],
                       kFirst ? 0.0f : L[2 * kStRows + t], d);
      }
    }
    const uint32_t ga = cnt.sa + i, stg = ga % kAStages;
    mbar_wait(&H->sa[stg], (ga / kAStages) & 1u, a.gs.err);
    if (s < P.se) {
      const int row = s * kSlice + P.lane;
      const int wlo = R0 + (i - kWinHalo) * kStRows;  // first row of the window
      const int wd = (kW > 0) ? kW : (int)((my1 - my0) >> 5);
      const float *ws;
      const int16_t *cs;
      const unsigned char *b = st_region(smem) + kA_Base + stg * kA_Bytes;
      if (kW > 0) {
        const int off = P.warp * kSlice * kW + (kW == 4 ? 4 * P.lane : P.lane);
        ws = reinterpret_cast<const float *>(b) + off;
        cs = reinterpret_cast<const int16_t *>(b + kA_C) + off;
      } else if (H->ok[stg]) {
        const int64_t off = my0 - H->base[stg];
        ws = reinterpret_cast<const float *>(b) + off + P.lane;
        cs = reinterpret_cast<const int16_t *>(b + kA_C) + off + P.lane;
      } else {
        ws = a.w32 + my0 + P.lane;
        cs = a.col16 + my0 + P.lane;
      }
      // p_hi at row k: from the ring when the window holds k, else formed
      // from global memory
      auto pat = [&](int k) -> float {
        if ((unsigned)(k - wlo) < (unsigned)kWinSpan) return ring[(k - R0) & (kPRingRows - 1)];
        FVC_CHK((unsigned)k < (unsigned)P.n, a.A.chk, kChkOffset, k = row);
        return kFirst ? a.z[k] : p_update(a.z[k], bh, bl, d.ph[k], d.pl[k]).x;
      };
      if (row < P.n) {
        const float pi = ring[(row - R0) & (kPRingRows - 1)];
        float t = myex * pi;
        if (kW == 4) {  // row-major stage: one 16-B and one 8-B shared load per row
          const float4 w4 = *reinterpret_cast<const float4 *>(ws);
          const uint2 c4 = *reinterpret_cast<const uint2 *>(cs);
          const float w[4] = {w4.x, w4.y, w4.z, w4.w};
          int c[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) c[k] = row + off16(c4, k);
#pragma unroll
          for (int k = 0; k < 4; ++k) t = fmaf(w[k], pi - pat(c[k]), t);
        } else if (kW > 0) {
          constexpr int W = kW > 0 ? kW : 1;
          int c[W];
          float w[W];
#pragma unroll
          for (int k = 0; k < kW; ++k) {
            c[k] = row + (int)cs[32 * k];
            w[k] = ws[32 * k];
          }
#pragma unroll
          for (int k = 0; k < kW; ++k) t = fmaf(w[k], pi - pat(c[k]), t);
        } else if (wd <= 4) {
          int c[4];
          float w[4], nb[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            c[k] = (k < wd) ? row + (int)cs[32 * k] : row;
            w[k] = (k < wd) ? ws[32 * k] : 0.0f;
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) nb[k] = pat(c[k]);
#pragma unroll
          for (int k = 0; k < 4; ++k) t = fmaf(w[k], pi - nb[k], t);
        } else {
          for (int k = 0; k < wd; ++k) t = fmaf(ws[32 * k], pi - pat(row + (int)cs[32 * k]), t);
        }
        a.q[row] = t;
        if (kFirst) a.e[row] = make_float2(0.0f, 0.0f);
        cpq.add(pi * t);
      }
    }
    my0 = n0;
    my1 = n1;
    myex = nex;
    __syncthreads();
  }
  if (jlast > kWinHalo) cnt.land += (uint32_t)(jlast - kWinHalo);
  cnt.sa += (uint32_t)nch;
  return cpq;
}

// Lane 0 of warp 0: bulk copies of phase-B chunk j into stage seq.
template <bool kPair, bool kUpdE>
__device__ __forceinline__ void issue_b(const MArgs &a, const MPart &P, unsigned char *smem,
                                        uint32_t seq, int j, const Dir &d) {
  StHdr *H = reinterpret_cast<StHdr *>(smem);
  const uint32_t stg = seq % kBStages;
  const int c0 = P.sb + kStChunkSlices * j;
  const int c1 = min(P.se, c0 + kStChunkSlices);
  const uint32_t rows = (uint32_t)(c1 - c0) * kSlice;
  const size_t r0 = (size_t)c0 * kSlice;
  unsigned char *b = st_region(smem) + stg * kB_Bytes;
  const uint32_t bytes = rows * 4u * (kPair ? 4u : 3u) + (kUpdE ? rows * 24u : 0u);
  uint64_t *bar = &H->sb[stg];
  mbar_arrive_expect_tx(bar, bytes);
  bulk_g2s(b + kB_Q, a.q + r0, rows * 4u, bar);
  bulk_g2s(b + kB_RS, a.rs + r0, rows * 4u, bar);
  if (kPair) bulk_g2s(b + kB_RSL, a.rsl + r0, rows * 4u, bar);
  bulk_g2s(b + kB_MINV, a.minv + r0, rows * 4u, bar);
  if (kUpdE) {
    bulk_g2s(b + kB_P1H, d.ph + r0, rows * 4u, bar);
    bulk_g2s(b + kB_P1L, d.pl + r0, rows * 4u, bar);
    bulk_g2s(b + kB_PVH, d.ch + r0, rows * 4u, bar);
    bulk_g2s(b + kB_PVL, d.cl + r0, rows * 4u, bar);
    bulk_g2s(b + kB_E, a.e + r0, rows * 8u, bar);
  }
}

// Lane 0 of warp 0: the first phase-B stages.  Every array they copy holds
// this block's own rows (written by this block before the __syncthreads
// that ended phase A) or constants, so they may be issued before the grid
// reduction that separates the phases, which then hides their latency.
template <bool kPair, bool kUpdE>
__device__ __forceinline__ void prefetch_b(const MArgs &a, const MPart &P, const Dir &d,
                                           unsigned char *smem, const StCount &cnt) {
  if (P.warp == 0 && P.lane == 0) {
    fence_proxy_async_global();
    fence_proxy_async_smem();
    const int nch = st_chunks(P);
    for (int j = 0; j < kBStages - 1 && j < nch; ++j)
      issue_b<kPair, kUpdE>(a, P, smem, cnt.sb + j, j, d);
  }
}

// The prefetched stages complete before the block may leave (a grid
// reduction that gave up): a bounded wait on each.
__device__ __forceinline__ void drain_prefetch_b(const MPart &P, unsigned char *smem,
                                                 const StCount &cnt) {
  StHdr *H = reinterpret_cast<StHdr *>(smem);
  const int nch = st_chunks(P);
  for (int j = 0; j < kBStages - 1 && j < nch; ++j) {
    const uint32_t seq = cnt.sb + (uint32_t)j;
    mbar_drain(&H->sb[seq % kBStages], (seq / kBStages) & 1u);
  }
}

// Staged phase B: the arithmetic of cg_phase_b, one row per thread.
// pre: prefetch_b has issued the first stages already
template <bool kPair, bool kUpdE>
__device__ __forceinline__ void cg_phase_b_st(const MArgs &a, const MPart &P, float a1,
                                              float a1_lo, float alpha, float alpha_lo,
                                              const Dir &d, CSum &crz, CSum &crr,
                                              unsigned char *smem, StCount &cnt, bool pre) {
  StHdr *H = reinterpret_cast<StHdr *>(smem);
  const int nch = st_chunks(P);
  if (!pre) prefetch_b<kPair, kUpdE>(a, P, d, smem, cnt);
  for (int i = 0; i < nch; ++i) {
    if (P.warp == 0 && P.lane == 0 && i + kBStages - 1 < nch)
      issue_b<kPair, kUpdE>(a, P, smem, cnt.sb + i + kBStages - 1, i + kBStages - 1, d);
    const uint32_t gi = cnt.sb + i, stg = gi % kBStages;
    mbar_wait(&H->sb[stg], (gi / kBStages) & 1u, a.gs.err);
    const int s = P.sb + kStChunkSlices * i + P.warp;
    const int row = s * kSlice + P.lane;
    if (s < P.se && row < P.n) {
      const float *b = reinterpret_cast<const float *>(st_region(smem) + stg * kB_Bytes);
      const int t = threadIdx.x;
      float2 eo;
      float ro, rlo = 0.0f, zo;
      cg_row_b<kPair, kUpdE>(
          a1, a1_lo, alpha, alpha_lo, b[kB_Q / 4 + t], b[kB_RS / 4 + t],
          kPair ? b[kB_RSL / 4 + t] : 0.0f, b[kB_MINV / 4 + t],
          kUpdE ? reinterpret_cast<const float2 *>(b + kB_E / 4)[t] : make_float2(0.0f, 0.0f),
          kUpdE ? b[kB_P1H / 4 + t] : 0.0f, kUpdE ? b[kB_P1L / 4 + t] : 0.0f,
          kUpdE ? b[kB_PVH / 4 + t] : 0.0f, kUpdE ? b[kB_PVL / 4 + t] : 0.0f, eo, ro, rlo, zo,
          crz, crr);
      if (kUpdE) a.e[row] = eo;
      a.rs[row] = ro;
      if (kPair) a.rsl[row] = rlo;
      a.z[row] = zo;
    }
    __syncthreads();
  }
  cnt.sb += (uint32_t)nch;
}

// The FP32 operator's 16-bit offsets no longer describe A (f32_bad, set
// by the build when a slot that held 0 at layout time now holds a far
// column's value): every block leaves before any work and the lead block
// reports FVC_ERR_UNSUPPORTED.  Every block reads the same word, written
// by the build earlier on the stream, so all take the same branch.
__device__ __forceinline__ bool f32_refused(const MArgs &a) {
  if (a.col16 == nullptr || a.f32_bad == nullptr || *a.f32_bad == 0) return false;
  if (mlead(a) && threadIdx.x == 0) {
    a.iresult[0] = 0;
    a.iresult[1] = FVC_ERR_UNSUPPORTED;
    a.iresult[2] = 0;
    a.result[2] = 0.0;
    a.result[3] = 0.0;
    a.result[4] = 0.0;
  }
  return true;
}

template <bool kStaged, int kW>
__device__ __forceinline__ void mixed_cg_body(const MArgs &a) {
  __shared__ double red[kMaxNV * 32];
  extern __shared__ __align__(128) unsigned char st_smem[];
  if (f32_refused(a)) return;
  const MPart P(a);
  StCount gch;  // staged copies issued so far, per ring
  if (kStaged) {
    if (threadIdx.x == 0) {
      StHdr *H = reinterpret_cast<StHdr *>(st_smem);
      for (int i = 0; i < kLandSlots; ++i) mbar_init(&H->land[i], 1);
      for (int i = 0; i < kAStages; ++i) mbar_init(&H->sa[i], 1);
      for (int i = 0; i < kBStages; ++i) mbar_init(&H->sb[i], 1);
      mbar_init_fence();
    }
    __syncthreads();
  }
  // FP64 scalars of the recurrence: kept by lane 0 of warp 0 in shared
  // memory (it runs all scalar FP64 work inside the all-reduces), read by
  // every thread after the all-reduce's closing __syncthreads
  __shared__ struct {
    double rz, rr_upd, relres, pend_alpha, alpha, rz_new;
    double bnorm2, scale, delta2, target2, res0;
    float alpha_f, alpha_lo, a1, a1_lo, beta, beta_lo;
    int action, status, updates;
  } sh;
  __shared__ float2 red2[kMaxNV * 32];
  enum { kContinue = 0, kUpdate = 1, kStop = 2 };
  unsigned int ep = 0;
  int it = 0;
  double res[4];
  if (!residual_sweep(a, ep, a.init != 0, res, red)) return;
  if (threadIdx.x == 0) {
    const double scale = (res[1] > 0.0) ? res[1] : 1.0;
    sh.bnorm2 = res[1];
    sh.scale = scale;
    sh.delta2 = a.inner_tol * a.inner_tol;
    sh.target2 = a.target * a.target * scale;
    sh.res0 = res[0];
    sh.relres = sqrt(res[0] / scale);
    sh.rz = res[2];
    sh.rr_upd = res[3];  // ||r||^2 (moving rows) at the last reliable update
    sh.pend_alpha = 0.0;
    sh.beta = 0.0f;
    sh.beta_lo = 0.0f;
    sh.updates = 0;
    sh.status = !(sh.relres == sh.relres) ? FVC_ERR_NAN
                : (sh.relres <= a.target) ? FVC_OK
                                          : FVC_ERR_NOCONV;
  }
  __syncthreads();
  int status = sh.status;
  float bh = 0.0f, bl = 0.0f;  // beta as an FP32 pair
  bool flip = false;           // which buffers hold p_prev / p this iteration
  bool pending = false;        // an alpha*p not yet added to e
  bool a_pre = false;          // the next phase A's first stages are in flight
  while (status == FVC_ERR_NOCONV && it < a.maxit) {
    ++it;
    Dir d;
    d.ph = flip ? a.pa : a.pb;
    d.pl = flip ? a.pal : a.pbl;
    d.ch = flip ? a.pb : a.pa;
    d.cl = flip ? a.pbl : a.pal;
    // p = z + beta p_prev (an FP32 pair); q = A p_hi; p_hi.q
    CSum pq[1];
    if (kStaged)
      pq[0] = (it == 1) ? cg_phase_a_st<true, kW>(a, P, bh, bl, d, st_smem, gch, a_pre)
                        : cg_phase_a_st<false, kW>(a, P, bh, bl, d, st_smem, gch, a_pre);
    else
      pq[0] = (it == 1) ? cg_phase_a<true>(a, P, bh, bl, d) : cg_phase_a<false>(a, P, bh, bl, d);
    a_pre = false;
    if (kStaged) {  // phase B's first copies before the wait
      if (pending)
        prefetch_b<true, true>(a, P, d, st_smem, gch);
      else
        prefetch_b<true, false>(a, P, d, st_smem, gch);
    }
    if (!grid_allreduce_ff<1>(a.gs, ep, pq, red2, [&](const double *t) {
          const double alpha_d = sh.rz / t[0];
          sh.alpha = alpha_d;
          sh.alpha_f = (float)alpha_d;
          sh.alpha_lo = (float)(alpha_d - (double)sh.alpha_f);
          sh.a1 = (float)sh.pend_alpha;
          sh.a1_lo = (float)(sh.pend_alpha - (double)sh.a1);
        })) {
      if (kStaged) drain_prefetch_b(P, st_smem, gch);
      return;
    }
    const float alpha = sh.alpha_f, alpha_lo = sh.alpha_lo;
    const float a1 = sh.a1, a1_lo = sh.a1_lo;
    // rs -= alpha q ; z = rs/m ; rs.z ; rs.rs ; every second iteration also
    // e += a_prev p_prev + alpha p (FP32 pair)
    CSum acc[2];
    if (kStaged) {
      if (pending)
        cg_phase_b_st<true, true>(a, P, a1, a1_lo, alpha, alpha_lo, d, acc[0], acc[1], st_smem,
                                  gch, true);
      else
        cg_phase_b_st<true, false>(a, P, a1, a1_lo, alpha, alpha_lo, d, acc[0], acc[1], st_smem,
                                   gch, true);
    } else if (pending) {
      cg_phase_b<true, true>(a, P, a1, a1_lo, alpha, alpha_lo, d, acc[0], acc[1]);
    } else {
      cg_phase_b<true, false>(a, P, a1, a1_lo, alpha, alpha_lo, d, acc[0], acc[1]);
    }
    const bool was_pending = pending;
    pending = !pending;
    if (kStaged && kW > 0) {  // the next phase A's first matrix stages before the wait
      prefetch_a<kW>(a, P, st_smem, gch);
      a_pre = true;
    }
    if (!grid_allreduce_ff<2>(a.gs, ep, acc, red2, [&](const double *t) {
          // the alpha*p of an iteration that did not update e is added later
          if (!was_pending) sh.pend_alpha = sh.alpha;
          const double rz_new = t[0];
          sh.rz_new = rz_new;
          if (mlead(a) && a.history && it <= kHistoryMax)
            a.history[it - 1] = (float)sqrt(t[1] / sh.scale);
          if (!(rz_new == rz_new)) {
            sh.status = FVC_ERR_NAN;
            sh.action = kStop;
          } else if (t[1] <= sh.delta2 * sh.rr_upd || t[1] <= sh.target2 || it >= a.maxit) {
            sh.action = kUpdate;
          } else {
            const double beta = rz_new / sh.rz;
            sh.beta = (float)beta;
            sh.beta_lo = (float)(beta - (double)sh.beta);
            sh.rz = rz_new;
            sh.action = kContinue;
          }
        })) {
      if (a_pre) drain_prefetch_a(P, st_smem, gch);
      return;
    }
    int action = sh.action;
    if (action == kUpdate) {
      // reliable update: fold e (and a deferred alpha p) into x, recompute
      // the true residual in FP64
      fold_correction(a, pending ? d.ch : nullptr, pending ? d.cl : nullptr, sh.pend_alpha);
      pending = false;
      if (!grid_barrier(a.gs, ep) || !residual_sweep(a, ep, false, res, red)) {
        if (a_pre) drain_prefetch_a(P, st_smem, gch);
        return;
      }
      if (threadIdx.x == 0) {
        const int u = ++sh.updates;
        const double relres = sqrt(res[0] / sh.scale);
        sh.res0 = res[0];
        sh.relres = relres;
        if (mlead(a) && a.trace && u <= kTraceMax) {
          a.trace[2 * (u - 1)] = (double)it;
          a.trace[2 * (u - 1) + 1] = relres;
        }
        sh.action = kContinue;
        if (!(relres == relres)) {
          sh.status = FVC_ERR_NAN;
          sh.action = kStop;
        } else if (relres <= a.target) {
          sh.status = FVC_OK;
          sh.action = kStop;
        } else {
          sh.rr_upd = res[3];
          // beta from the replaced (true) residual, or with update_beta from
          // the recursive one; the next alpha uses the true r.z
          const double beta = (a.update_beta ? sh.rz_new : res[2]) / sh.rz;
          sh.beta = (float)beta;
          sh.beta_lo = (float)(beta - (double)sh.beta);
          sh.rz = res[2];
        }
        sh.pend_alpha = 0.0;
      }
      __syncthreads();
      action = sh.action;
    }
    if (action == kStop) {
      status = sh.status;
      break;
    }
    bh = sh.beta;
    bl = sh.beta_lo;
    flip = !flip;
  }
  if (a_pre) drain_prefetch_a(P, st_smem, gch);
  if (mlead(a) && threadIdx.x == 0) {
    a.iresult[0] = sh.updates;
    a.iresult[1] = (status == FVC_ERR_NOCONV) ? sh.status : status;
    a.iresult[2] = it;
    a.result[2] = sh.relres;
    a.result[3] = sh.res0;
    a.result[4] = sh.bnorm2;
  }
}

__global__ void __launch_bounds__(1024, 1) mixed_cg(MArgs a) { mixed_cg_body<false, 0>(a); }

// Staged forms: 1024 threads, kStSmem bytes of dynamic shared memory, and
// the 16-bit column offsets (col16) present; _w3/_w4 when every slice has
// width 3 / 4 in the padded uniform layout (ell_w; cells of triangle /
// quadrilateral meshes).
__global__ void __launch_bounds__(1024, 1) mixed_cg_staged(MArgs a) { mixed_cg_body<true, 0>(a); }
__global__ void __launch_bounds__(1024, 1) mixed_cg_staged_w3(MArgs a) {
  mixed_cg_body<true, 3>(a);
}
__global__ void __launch_bounds__(1024, 1) mixed_cg_staged_w4(MArgs a) {
  mixed_cg_body<true, 4>(a);
}

// The reference's Jacobi BiCGSTAB (Iterativos.f:140-234) in FP32 on the
// correction equation A e = r, inside FP64 defect correction.
constexpr int kBcgStall = 100;
constexpr int kSweepStall = 3;

__device__ __forceinline__ void mixed_bicgstab_body(const MArgs &a) {
  __shared__ double red[kMaxNV * 32];
  __shared__ float2 red2[kMaxNV * 32];
  // the inner iteration's scalars: FP64 work of lane 0 of warp 0 inside the
  // all-reduces (GB300 runs FP64 at ~1/64 of the FP32 rate: three FP64
  // divisions in every thread of every iteration kept the FP64 pipe 40%
  // busy), handed to the block as FP32 through shared memory
  __shared__ struct {
    double rr0, best;
    float alpha, omega, beta;
    int it_best, go;
  } bs;
  if (f32_refused(a)) return;
  const MPart P(a);
  unsigned int ep = 0;
  int sweep = 0, inner_total = 0, status = FVC_ERR_NOCONV;
  double res[4];
  double relres = 0.0, bnorm2 = 0.0, best_rel = 0.0;
  int flat = 0;
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
    // sweeps that no longer cut the FP64 residual by a tenth (the FP32
    // operator's rounding outweighs the correction): after kSweepStall of
    // them in a row the solve stops early with FVC_ERR_NOCONV, below both
    // max_refine and maxit (every block sees the same relres)
    if (sweep == 0 || relres <= 0.9 * best_rel) {
      flat = 0;
    } else if (++flat >= kSweepStall) {
      break;
    }
    best_rel = (sweep == 0) ? relres : fmin(best_rel, relres);
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
    if (threadIdx.x == 0) {
      bs.best = fabs(d);
      bs.it_best = 0;
    }
    int it = 0;
    for (;;) {
      ++it;
      // v = A z ; rr0 = s.r0 ; v.r0
      CSum c01[2];
      mfor_rows2(P, [&](const int(&sl)[2], const int(&rw)[2], const bool(&ok)[2]) {
        float vi[2], r0i[2], si[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          vi[u] = arow32(a, sl[u], P.lane, rw[u], [&](int k) { return z[k]; });
          r0i[u] = r0[rw[u]];
          si[u] = sv[rw[u]];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
          if (ok[u]) {
            v[rw[u]] = vi[u];
            c01[0].add(si[u] * r0i[u]);
            c01[1].add(vi[u] * r0i[u]);
          }
      });
      // breakdown (v.r0 or r0.s vanished in FP32): leave the correction as it
      // is and restart from an FP64 residual in the next sweep
      if (!grid_allreduce_ff<2>(a.gs, ep, c01, red2, [&](const double *q) {
            bs.rr0 = q[0];
            bs.alpha = (float)(q[0] / q[1]);
            bs.go = (isfinite(bs.alpha) && bs.alpha != 0.0f) ? 1 : 0;
          }))
        return;
      if (!bs.go) break;
      const float alpha = bs.alpha;
      // e += alpha z ; s -= alpha v ; z = s/m
      mfor_rows2(P, [&](const int(&sl)[2], const int(&rw)[2], const bool(&ok)[2]) {
        float2 ev[2];
        float zi[2], vv[2], si[2], mi[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          ev[u] = e[rw[u]];
          zi[u] = z[rw[u]];
          vv[u] = v[rw[u]];
          si[u] = sv[rw[u]];
          mi[u] = minv[rw[u]];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
          if (ok[u]) {
            e[rw[u]] = df_axpy(ev[u], alpha, 0.0f, zi[u]);
            const float sn = fmaf(-alpha, vv[u], si[u]);
            sv[rw[u]] = sn;
            z[rw[u]] = sn * mi[u];
          }
      });
      if (!grid_barrier(a.gs, ep)) return;
      // t = A z ; t.s ; t.t
      CSum c23[2];
      mfor_rows2(P, [&](const int(&sl)[2], const int(&rw)[2], const bool(&ok)[2]) {
        float ti[2], si[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          ti[u] = arow32(a, sl[u], P.lane, rw[u], [&](int k) { return z[k]; });
          si[u] = sv[rw[u]];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
          if (ok[u]) {
            t[rw[u]] = ti[u];
            c23[0].add(ti[u] * si[u]);
            c23[1].add(ti[u] * ti[u]);
          }
      });
      if (!grid_allreduce_ff<2>(a.gs, ep, c23, red2, [&](const double *q) {
            bs.omega = (q[1] > 0.0) ? (float)(q[0] / q[1]) : 0.0f;
            bs.go = isfinite(bs.omega) ? 1 : 0;
          }))
        return;
      if (!bs.go) break;
      const float omega = bs.omega;
      // e += w z ; s -= w t ; s.z ; r0.s
      CSum c45[2];
      mfor_rows2(P, [&](const int(&sl)[2], const int(&rw)[2], const bool(&ok)[2]) {
        float2 ev[2];
        float zi[2], ti[2], si[2], r0i[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          ev[u] = e[rw[u]];
          zi[u] = z[rw[u]];
          ti[u] = t[rw[u]];
          si[u] = sv[rw[u]];
          r0i[u] = r0[rw[u]];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
          if (ok[u]) {
            e[rw[u]] = df_axpy(ev[u], omega, 0.0f, zi[u]);
            const float sn = fmaf(-omega, ti[u], si[u]);
            sv[rw[u]] = sn;
            c45[0].add(sn * zi[u]);
            c45[1].add(r0i[u] * sn);
          }
      });
      // stop on the inner reduction, a NaN, maxit or w = 0; restarted
      // BiCGSTAB: an inner solve whose residual has not improved for
      // kBcgStall iterations (FP32 stagnation) restarts from an FP64 one
      if (!grid_allreduce_ff<2>(a.gs, ep, c45, red2, [&](const double *q) {
            const double sz = fabs(q[0]);
            int go = 1;
            if (!(q[0] == q[0]) || sz <= stop2 || inner_total + it >= a.maxit ||
                bs.omega == 0.0f) {
              go = 0;
            } else if (sz < 0.99 * bs.best) {
              bs.best = sz;
              bs.it_best = it;
            } else if (it - bs.it_best > kBcgStall) {
              go = 0;
            }
            bs.beta = (float)((q[1] / bs.rr0) * ((double)bs.alpha / (double)bs.omega));
            bs.go = go;
          }))
        return;
      if (!bs.go) break;
      const float beta = bs.beta;
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
  if (mlead(a) && threadIdx.x == 0) {
    a.iresult[0] = sweep;
    a.iresult[1] = status;
    a.iresult[2] = inner_total;
    a.result[2] = relres;
    a.result[3] = res[0];
    a.result[4] = bnorm2;
  }
}

__global__ void __launch_bounds__(1024, 1) mixed_bicgstab(MArgs a) { mixed_bicgstab_body(a); }

// Batched mixed-precision solves: every block runs the mixed CG (code 1)
// or the mixed BiCGSTAB (code 2) of its system of the block-diagonal
// matrix, on that system's slices and synchronisation state: a group of
// blocks of one cooperative launch, or (d.gs.cluster) one thread-block
// cluster of an ordinary launch.
template <int kMaxT>
__global__ void __launch_bounds__(kMaxT, 1024 / kMaxT)
    mixed_batched(MArgs a, const BatchSys *__restrict__ sys, const int *__restrict__ sob) {
  const BatchSys d = sys[sob[blockIdx.x]];
  if (batch_masked(d, blockIdx.x == d.gs.base)) return;
  MArgs am = a;
  am.gs = d.gs;
  am.grp_s0 = d.s0;
  am.grp_s1 = d.s1;
  am.grp_nb = (int)d.gs.nblocks;
  am.grp_base = (int)d.gs.base;
  am.target = d.tol;
  am.inner_tol = d.inner_tol;
  am.init = d.init;
  am.result = d.result;
  am.iresult = d.iresult;
  am.trace = nullptr;
  am.history = nullptr;
  if (d.code == 2) {
    am.rsl = nullptr;
    mixed_bicgstab_body(am);
  } else {
    mixed_cg_body<false, 0>(am);
  }
  cluster_close(d.gs);
}

// The launch-wide arguments of the mixed kernels over matrix A and the
// FP32 vectors of S (rsl, gs and the solve's scalars are the caller's).
MArgs mixed_args(const DeviceMatrix &A, const Scratch &S, const double *b, double *x) {
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
  a.col16 = A.col16_ok ? A.col16 : nullptr;
  a.ell_w = A.ell_w;
  a.A.chk = check_word(S);
  a.sflag = A.sflag;
  a.f32_bad = A.f32_bad;
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
  a.rsl = S.f[9];
  a.pal = S.f[5];  // CG only (BiCGSTAB uses these buffers as r0 and t)
  a.pbl = S.f[6];
  return a;
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

int32_t ensure_f32_vectors(Scratch &S, size_t n) {
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
  return FVC_OK;
}

const void *mixed_batched_kernel(int threads) {
  return threads <= 128   ? (const void *)mixed_batched<128>
         : threads <= 256 ? (const void *)mixed_batched<256>
                          : (const void *)mixed_batched<1024>;
}

int32_t launch_mixed_batched(const DeviceMatrix &A, const Scratch &S, const BatchSys *dsys,
                             const int *dsob, int blocks, int threads, int cluster,
                             const double *b, double *x, int maxit, const fvc_opts &o,
                             cudaStream_t stream) {
  MArgs a = mixed_args(A, S, b, x);
  a.max_refine = (o.max_refine > 0) ? o.max_refine : 30;
  a.update_beta = o.update_beta;
  a.maxit = maxit;
  // (the shared-memory carveout stays at its default: the caller sized the
  // grid by the occupancy under it)
  const void *kern = mixed_batched_kernel(threads);
  void *args[] = {&a, &dsys, &dsob};
  const cudaError_t ce = launch_groups(kern, blocks, threads, cluster, args, stream);
  count_launch();
  if (ce != cudaSuccess) {
    fprintf(stderr, "fvcgpu: batched mixed launch failed: %s\n", cudaGetErrorString(ce));
    return FVC_ERR_CUDA;
  }
  return FVC_OK;
}

// The FP32 operator: its layout (16-bit offsets, uniform width) once per
// structure, with a host wait; then, after every value upload, the values
// alone, stream-ordered (so that a captured graph can rebuild them).
int32_t build_f32_copy(DeviceMatrix &A, cudaStream_t stream, int mode) {
  if (A.layout32 && A.layout_mode != mode) {
    // the other slice-width choice: the operator is laid out anew (its
    // slot arrays have another size)
    if (cudaStreamSynchronize(stream) != cudaSuccess) return FVC_ERR_CUDA;
    cudaFree(A.val32);
    cudaFree(A.col16);
    A.val32 = nullptr;
    A.col16 = nullptr;
    A.layout32 = false;
    A.have32 = false;
  }
  if (A.have32) return FVC_OK;
  int blocks = std::max(1, std::min((A.nslices + 7) / 8, sm_count_m() * 8));
  if (A.layout32) {
    if (cudaMemsetAsync(A.f32_bad, 0, sizeof(int), stream) != cudaSuccess) return FVC_ERR_CUDA;
    build_f32_operator<<<blocks, 256, 0, stream>>>(A.n, A.nslices, A.sptr, A.col, A.val, A.jac,
                                                   A.val32, A.diag32, A.minv32, A.col16,
                                                   A.sflag, A.ell_w, A.col16_ok ? 1 : 0,
                                                   A.f32_bad);
    count_launch();
    if (cudaPeekAtLastError() != cudaSuccess) return FVC_ERR_CUDA;
    A.have32 = true;
    return FVC_OK;
  }
  int *flags = nullptr;  // [0] a column offset overflows 16 bits, [1] min, [2] max slice width
  if (cudaMalloc(&flags, 3 * sizeof(int)) != cudaSuccess) return FVC_ERR_CUDA;
  const int init[3] = {0, 1 << 30, 0};
  cudaMemcpyAsync(flags, init, sizeof(init), cudaMemcpyHostToDevice, stream);
  scan_slices<<<blocks, 256, 0, stream>>>(A.n, A.nslices, A.sptr, A.col, A.val, flags);
  count_launch();
  int hf[3] = {1, 0, 0};
  cudaMemcpyAsync(hf, flags, sizeof(hf), cudaMemcpyDeviceToHost, stream);
  cudaError_t ce = cudaStreamSynchronize(stream);
  cudaFree(flags);
  if (ce != cudaSuccess) return FVC_ERR_CUDA;
  A.col16_ok = (hf[0] == 0);
  // slices at most 4 wide (the cells of triangle / quadrilateral meshes):
  // pad them all to the widest, so the staged kernel needs no slice pointers
  A.ell_w = (mode == 0 && A.col16_ok && A.nslices > 0 && hf[2] >= 3 && hf[2] <= 4) ? hf[2] : 0;
  A.layout_mode = mode;
  const size_t sl = std::max<size_t>(
      1, A.ell_w > 0 ? (size_t)A.nslices * kSlice * A.ell_w : (size_t)A.slots);
  if (!A.val32 && cudaMalloc(&A.val32, sizeof(float) * sl) != cudaSuccess) return FVC_ERR_CUDA;
  // row arrays cover whole slices (the staged loops copy 32-row units)
  const size_t nrow = (size_t)A.nslices * kSlice + 64;
  if (!A.diag32 && cudaMalloc(&A.diag32, sizeof(float) * nrow) != cudaSuccess)
    return FVC_ERR_CUDA;
  if (!A.minv32 && cudaMalloc(&A.minv32, sizeof(float) * nrow) != cudaSuccess)
    return FVC_ERR_CUDA;
  if (!A.col16 && cudaMalloc(&A.col16, sizeof(int16_t) * sl) != cudaSuccess) return FVC_ERR_CUDA;
  if (!A.sflag && cudaMalloc(&A.sflag, (size_t)A.nslices + 1) != cudaSuccess) return FVC_ERR_CUDA;
  if (!A.f32_bad && cudaMalloc(&A.f32_bad, sizeof(int)) != cudaSuccess) return FVC_ERR_CUDA;
  if (cudaMemsetAsync(A.f32_bad, 0, sizeof(int), stream) != cudaSuccess) return FVC_ERR_CUDA;
  build_f32_operator<<<blocks, 256, 0, stream>>>(A.n, A.nslices, A.sptr, A.col, A.val, A.jac,
                                                 A.val32, A.diag32, A.minv32, A.col16, A.sflag,
                                                 A.ell_w, A.col16_ok ? 1 : 0, A.f32_bad);
  count_launch();
  ce = cudaStreamSynchronize(stream);
  if (ce != cudaSuccess) return FVC_ERR_CUDA;
  A.layout32 = true;
  A.have32 = true;
  return FVC_OK;
}

int32_t enqueue_mixed(const DeviceMatrix &A0, Scratch &S, int code, const double *b, double *x,
                      double tol, int maxit, int init, const fvc_opts &o, cudaStream_t stream,
                      bool launch) {
  DeviceMatrix &A = const_cast<DeviceMatrix &>(A0);
  if (code != 1 && code != 2) return FVC_ERR_UNSUPPORTED;
  int32_t rc = build_f32_copy(A, stream, o.fp32_layout);
  if (rc != FVC_OK) return rc;
  if ((rc = ensure_f32_vectors(S, (size_t)A.n)) != FVC_OK) return rc;
  const int threads = block_threads_for(o.block_threads, A.nslices, sm_count_m());
  // CG streams through shared-memory stages when its layout allows and
  // each block owns enough 1024-row chunks to fill the pipeline beside its
  // +-3-chunk window; below, plain loads are faster (per iteration on
  // GB300, staged vs plain: 262k rows 16.5 vs 14.1 us, 1.05M 28.9 vs
  // 28.6 us, 4.19M 87 vs 122 us)
  const bool staged = code == 1 && threads == kStRows && A.col16_ok &&
                      (o.staging == 2 || (o.staging == 0 && A.n >= kStagedRows));
  auto kern = (code != 1) ? mixed_bicgstab
              : !staged        ? mixed_cg
              : A.ell_w == 4   ? mixed_cg_staged_w4
              : A.ell_w == 3   ? mixed_cg_staged_w3
                               : mixed_cg_staged;
  const size_t dsmem = staged ? kStSmem : 0;
  if (staged) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem) !=
        cudaSuccess)
      return FVC_ERR_CUDA;
  } else {
    // the plain-load kernels gather through L1: keep it at its largest
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  }
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, dsmem);
  if (occ <= 0) occ = 1;
  if (o.blocks_per_sm > 0 && o.blocks_per_sm < occ) occ = o.blocks_per_sm;
  const int warps = threads / 32;
  int blocks = std::max(1, std::min(occ * sm_count_m(), (A.nslices + warps - 1) / warps));
  if (o.max_blocks > 0) blocks = std::min(blocks, o.max_blocks);
  if (ensure_sync(S, (size_t)blocks) != FVC_OK) return FVC_ERR_CUDA;
  if (!launch) return FVC_OK;
  reset_sync(S, stream);
  MArgs a = mixed_args(A, S, b, x);
  a.rsl = (code == 1) ? S.f[9] : nullptr;
  a.gs = make_sync(S, blocks);
  a.target = (o.refine_tol > 0) ? o.refine_tol : tol;
  a.inner_tol = (o.inner_tol > 0) ? o.inner_tol : kInnerTolDefault;
  a.max_refine = (o.max_refine > 0) ? o.max_refine : 30;
  a.update_beta = o.update_beta;
  a.maxit = maxit;
  a.init = init;
  a.result = S.result;
  a.iresult = S.iresult;
  a.trace = S.trace;
  a.history = S.history;
  void *args[] = {&a};
  const cudaError_t ce =
      cudaLaunchCooperativeKernel((const void *)kern, dim3(blocks), dim3(threads), args, dsmem, stream);
  count_launch();
  if (ce != cudaSuccess) {
    fprintf(stderr, "fvcgpu: cooperative launch failed: %s\n", cudaGetErrorString(ce));
    return FVC_ERR_CUDA;
  }
  return FVC_OK;
}

int32_t run_mixed(const DeviceMatrix &A, Scratch &S, int code, const double *b, double *x,
                  double tol, int maxit, int init, const fvc_opts &o, cudaStream_t stream,
                  fvc_stats *st) {
  // FP64 BiCGSTAB to the mixed solve's target on ||r||2/||b||2 (stats: the
  // FP32 part's iterations and sweeps kept, both parts' times summed)
  const double target = (o.refine_tol > 0) ? o.refine_tol : tol;
  auto fp64_bicgstab = [&](int from_init, int its_left, int fp32_its, int sweeps, float ms0) {
    fvc_opts fo = o;
    fo.precision = FVC_PREC_FP64;
    fo.stop_rule = 1;
    fo.want_residual = 1;
    fvc_stats s2{};
    const int32_t rc2 = run_bicgstab(A, S, b, x, target, its_left, from_init, fo, stream, &s2);
    if (st) {
      *st = s2;
      st->status = rc2;
      st->iterations = fp32_its + s2.iterations;
      st->inner_iterations = fp32_its;
      st->refinements = sweeps;
      st->conv = target;
      st->solve_ms = ms0 + s2.solve_ms;
    }
    return rc2;
  };
  if (code == 2 && A.bcg32_stalled) return fp64_bicgstab(init, maxit, 0, 0, 0.f);
  // allocations (and the FP32 layout) before the timed launch
  int32_t rc = enqueue_mixed(A, S, code, b, x, tol, maxit, init, o, stream, false);
  if (rc != FVC_OK) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, stream);
  rc = enqueue_mixed(A, S, code, b, x, tol, maxit, init, o, stream, true);
  cudaEventRecord(e1, stream);
  if (rc != FVC_OK) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  double res[16];
  int ires[16], err = 0;
  cudaMemcpyAsync(res, S.result, sizeof(res), cudaMemcpyDeviceToHost, stream);
  cudaMemcpyAsync(ires, S.iresult, sizeof(ires), cudaMemcpyDeviceToHost, stream);
  cudaMemcpyAsync(&err, S.err, sizeof(int), cudaMemcpyDeviceToHost, stream);
  const cudaError_t ce = cudaStreamSynchronize(stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ce != cudaSuccess) return FVC_ERR_CUDA;
  if (err != 0) return FVC_ERR_TIMEOUT;
  if (const int32_t c = check_word_status(S, stream); c != FVC_OK) return c;
  if (ires[1] == FVC_ERR_UNSUPPORTED)
    fprintf(stderr,
            "fvcgpu: mixed solve refused: a matrix slot that held 0 when the FP32 layout was "
            "chosen now holds a value whose column is more than 32767 rows away; set the "
            "matrix again (fvc_matrix_set) to lay the FP32 operator out anew\n");
  if (st) {
    st->status = ires[1];
    st->iterations = ires[2];
    st->inner_iterations = ires[2];
    st->refinements = ires[0];  // CG: reliable updates; BiCGSTAB: sweeps
    st->energy = 0.0;
    st->conv = target;
    st->final_crit = res[2];
    st->rel_residual = res[2];
    st->solve_ms = ms;
  }
  const int max_refine = (o.max_refine > 0) ? o.max_refine : 30;
  if (code == 2 && ires[1] == FVC_ERR_NOCONV && ires[0] < max_refine && ires[2] < maxit) {
    // the defect-correction sweeps stalled (stopped early by the kernel):
    // FP64 finishes from the current iterate with the iterations left, and
    // later mixed BiCGSTAB solves of this structure start in FP64
    A.bcg32_stalled = true;
    return fp64_bicgstab(0, maxit - ires[2], ires[2], ires[0], ms);
  }
  return ires[1];
}

}  // namespace fvc
