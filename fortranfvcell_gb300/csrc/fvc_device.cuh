// fvc_device.cuh -- device-side building blocks shared by the SpMV and
// Krylov kernels of libfvcgpu (sm_103a).
//
// Matrix layout on the device: sliced ELLPACK with slice height 32
// (SELL-32).  Slice s covers rows [32s, 32s+32); its width w_s is the
// longest row of the slice; entry k of lane l sits at slot
// slice_ptr[s] + 32*k + l, so one warp reads one slice with fully
// coalesced 32-bit (columns) and 64-bit (values) streams.  Padding slots
// hold column = own row and value = 0, which leaves every sum unchanged.
// Row entries keep the reference's per-row order, and the diagonal is
// applied first or last exactly where src/Matvec.f applies it, so the
// FP64 SpMV is bit-identical to the reference routine (no FMA contraction:
// products and sums are rounded separately, as the Fortran loops do).
#pragma once
#include <cooperative_groups.h>
#include <cstdint>
#include <cuda_runtime.h>

#include "fvc_internal.h"

namespace fvc {

constexpr int kSlice = 32;

template <typename V>
struct SellView {
  int n;                 // rows
  int nslices;
  const int64_t *sptr;   // nslices+1 slot offsets
  const int *col;        // 0-based columns
  const V *val;          // values (negated off-diagonals, as stored)
  const V *diag;         // n (null for DIAG_NONE)
  int diag_mode;
  const int *mirror = nullptr;  // per slot: the slot of the transposed entry
                                // (symmetric patterns; transposed solves only)
  int *chk = nullptr;           // check builds: the launch's error word
};

// Opt-in device checks (compiled with -DFVC_CHECK, the library's check
// variant; see build.py).  A column, slice width, offset or mirror index
// outside its array is recorded in an error word -- the first failing
// check's code, kept by atomicCAS -- and the access is redirected to a safe
// index (the row itself, or an empty slice), so nothing is read out of
// bounds and nothing traps.  The word is the launch's grid-wait error word:
// every grid wait sees it and returns, so the launch ends through its
// normal error path, and the host reports FVC_ERR_ARG with the check's
// name (check_status).  Without FVC_CHECK the checks compile to nothing.
enum CheckCode : int {
  kChkColumn = 101,      // SELL column outside [0, n)
  kChkSliceWidth = 102,  // slice width negative or above n
  kChkOffset = 103,      // FP32 operator: row + 16-bit offset outside [0, n)
  kChkMirror = 104,      // transposed solves: mirror slot outside the slots
  kChkCluster = 105,     // cluster PCG: a column whose owner CTA is not in the cluster
};
#ifdef FVC_CHECK
#define FVC_CHK(cond, word, code, fix)                        \
  do {                                                        \
    if (!(cond)) {                                            \
      int *w_ = (word);                                       \
      if (w_) atomicCAS(w_, 0, (int)(code));                  \
      fix;                                                    \
    }                                                         \
  } while (0)
#else
#define FVC_CHK(cond, word, code, fix) \
  do {                                 \
  } while (0)
#endif

// Grid synchronisation state of one persistent launch.  `count` is a
// monotonically increasing arrival counter (episode e completes when it
// reaches e * nblocks, so it never needs resetting inside the launch);
// `flag` holds the last released episode.  Partials and totals rotate over
// four slots so a block running ahead never overwrites data still read.
struct GridSync {
  unsigned int *count;
  unsigned int *flag;
  int *err;                // sticky error (FVC_ERR_TIMEOUT on a stuck wait)
  double *partials;        // 4 slots x kMaxNV x nblocks
  double *totals;          // 4 slots x kMaxNV
  unsigned int nblocks;    // blocks that synchronise through this state
  unsigned int base;       // blockIdx.x of the first of them (0 for a whole grid)
  // nonzero: the nblocks blocks are one thread-block cluster; the waits
  // and reductions below then use the cluster barrier and distributed
  // shared memory instead of global memory (cluster_exchange)
  int cluster = 0;
};

constexpr int kMaxNV = 4;

// The cluster form of a reduction.  Lane 0 of warp 0 of every CTA has
// stored its block's NV partials in its own slot (mine); every thread of
// every CTA then meets at the cluster barrier (arrive.release /
// wait.acquire at cluster scope: the slots, and every global-memory write
// made before it, are visible to the whole cluster after it); warp 0 reads
// the CTAs' slots in rank order through distributed shared memory and sums
// them in a fixed shuffle tree, so every CTA holds identical totals (in lane
// 0 of warp 0).  There is no spin-wait: the barrier is the hardware's, and
// every CTA reaches it the same number of times because every branch
// around it depends only on those identical totals.  Two slots alternate
// (a slot is written again only after a later barrier, so never while a
// CTA still reads it), and the kernel ends with one more barrier so that
// no CTA's shared memory goes away while another reads it.
template <int NV>
__device__ __forceinline__ void cluster_exchange(double (*slots)[kMaxNV], unsigned int ep,
                                                 double (&t)[NV > 0 ? NV : 1]) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  cl.sync();
  if (NV > 0 && threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int nb = (int)cl.num_blocks();
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double u = (lane < nb) ? *cl.map_shared_rank(&slots[ep & 1u][q], lane) : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) u = __dadd_rn(u, __shfl_down_sync(0xffffffffu, u, o));
      t[q] = u;
    }
  }
}

// the closing barrier of a kernel whose blocks reduce through cluster_exchange
__device__ __forceinline__ void cluster_close(const GridSync &gs) {
  if (gs.cluster) cooperative_groups::this_cluster().sync();
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int atom_add_acq_rel(unsigned int *p, unsigned int v) {
  unsigned int old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ void red_add_release(unsigned int *p, unsigned int v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release(unsigned int *p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Every wait is bounded: after kBarrierTimeoutNs the block records
// FVC_ERR_TIMEOUT and leaves; the other waiters see the flag and leave too,
// so a broken launch returns an error instead of spinning.
constexpr uint64_t kBarrierTimeoutNs = 4000000000ull;  // 4 s

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum of NV values per thread; result valid in thread 0.
// Fixed tree order -> deterministic.  red must hold NV*32 doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = warp_sum(v[q]);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; ++q) red[q * 32 + warp] = v[q];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double t = (lane < nwarps) ? red[q * 32 + lane] : 0.0;
      v[q] = warp_sum(t);
    }
  }
  __syncthreads();
}

// Grid-wide barrier (NV == 0) or deterministic all-reduce of NV doubles
// per thread.  One arrival atomic per block; the last block to arrive sums
// the per-block partials in block order (the same order whichever block is
// last) and releases the others, which then read the NV totals.  Returns
// false, with gs.err set, when a wait exceeded its bound.
template <int NV>
__device__ __forceinline__ bool grid_allreduce(const GridSync &gs, unsigned int &episode,
                                               double (&v)[NV > 0 ? NV : 1], double *red) {
  __shared__ int s_last, s_ok;
  if (NV > 0) {
    block_sum<(NV > 0 ? NV : 1)>(v, red);
  } else {
    __syncthreads();
  }
  if (gs.cluster) {
    __shared__ double s_slot[2][kMaxNV];
    const unsigned int ep = ++episode;
    if (NV > 0 && threadIdx.x == 0)
#pragma unroll
      for (int q = 0; q < NV; ++q) s_slot[ep & 1u][q] = v[q];
    double t[NV > 0 ? NV : 1];
    cluster_exchange<NV>(s_slot, ep, t);
    if (NV > 0) {
      if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) red[q] = t[q];
      __syncthreads();
#pragma unroll
      for (int q = 0; q < NV; ++q) v[q] = red[q];
      __syncthreads();
    }
    return true;
  }
  if (gs.nblocks == 1) {  // one block: its sum is the total (same value)
    ++episode;
    if (NV > 0) {
      if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) red[q] = v[q];
      __syncthreads();
#pragma unroll
      for (int q = 0; q < NV; ++q) v[q] = red[q];
      __syncthreads();
    }
    return true;
  }
  const unsigned int ep = ++episode;
  const unsigned int nb = gs.nblocks;
  double *part = gs.partials + (size_t)(ep & 3u) * kMaxNV * nb;
  double *tot = gs.totals + (ep & 3u) * kMaxNV;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) part[(size_t)q * nb + (blockIdx.x - gs.base)] = v[q];
    const unsigned int old = atom_add_acq_rel(gs.count, 1u);
    s_last = (old == ep * nb - 1u);
    s_ok = 1;
  }
  __syncthreads();
  if (s_last) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (NV > 0 && warp < NV) {
      const double *p = part + (size_t)warp * nb;
      double t = 0.0;
      for (unsigned int b = lane; b < nb; b += 32) t = __dadd_rn(t, __ldcg(p + b));
      t = warp_sum(t);
      if (lane == 0) __stcg(tot + warp, t);
    }
    __syncthreads();
    if (threadIdx.x == 0) st_release(gs.flag, ep);
  } else if (threadIdx.x == 0) {
    const uint64_t t0 = global_ns();
    unsigned int spins = 0;
    while (ld_acquire(gs.flag) < ep) {
      if (*(volatile int *)gs.err != 0) {
        s_ok = 0;
        break;
      }
      if ((++spins & 255u) == 0 && global_ns() - t0 > kBarrierTimeoutNs) {
        atomicExch(gs.err, 7 /* FVC_ERR_TIMEOUT */);
        s_ok = 0;
        break;
      }
      __nanosleep(20);
    }
  }
  __syncthreads();
  if (!s_ok) return false;
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = __ldcg(tot + q);
  return true;
}

// Grid-wide deterministic sum of NV FP64 values per thread, for the FP64
// solvers.  GB300 issues FP64 at ~2 lanes per clock per SM, so the block
// sum avoids a butterfly in every warp (5 x 32 lanes x 32 warps adds):
// the values go to shared memory (buf: NV x blockDim doubles), four warps
// (one per SM sub-partition) add 8 values per lane each, warp 0 adds those
// and finishes with a shuffle tree -- a fixed order, about 2.5x fewer FP64
// instructions (blockDim.x must be a multiple of 128).  The block's
// partial is published with a release add on the grid counter; every block waits for all arrivals and sums all
// partials in block order itself.  Lane 0 of warp 0 then calls f(totals)
// -- the place for the iteration's scalar FP64 work (one thread instead of
// 1024) -- and one __syncthreads hands its results (through shared memory)
// to the block.  Returns false when a wait exceeded its bound (gs.err set).
template <int NV, typename F>
__device__ __forceinline__ bool grid_allreduce_d(const GridSync &gs, unsigned int &episode,
                                                 const double (&v)[NV], double *buf, F &&f) {
  __shared__ int s_ok;
  __shared__ double s_part[NV][128];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bd = blockDim.x, per = bd >> 7;  // values per lane of the first level
#pragma unroll
  for (int q = 0; q < NV; ++q) buf[q * bd + threadIdx.x] = v[q];
  if (threadIdx.x == 0) s_ok = 1;
  __syncthreads();
  if (warp < 4) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const double *b = buf + q * bd + warp * (bd >> 2) + lane;
      double u = b[0];
      for (int k = 1; k < per; ++k) u = __dadd_rn(u, b[32 * k]);
      s_part[q][warp * 32 + lane] = u;
    }
  }
  __syncthreads();
  const unsigned int ep = ++episode;
  if (gs.cluster) {
    __shared__ double s_slot[2][kMaxNV];
    if (warp == 0) {
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        double u = s_part[q][lane];
#pragma unroll
        for (int k = 1; k < 4; ++k) u = __dadd_rn(u, s_part[q][32 * k + lane]);
        u = warp_sum(u);
        if (lane == 0) s_slot[ep & 1u][q] = u;
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
      double u = s_part[q][lane];
#pragma unroll
      for (int k = 1; k < 4; ++k) u = __dadd_rn(u, s_part[q][32 * k + lane]);
      bsum[q] = warp_sum(u);
    }
    bool ok = true;
    double t[NV];
    if (nb == 1) {  // one block: its sum is the total (same value)
#pragma unroll
      for (int q = 0; q < NV; ++q) t[q] = bsum[q];
    } else {
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

__device__ __forceinline__ bool grid_barrier(const GridSync &gs, unsigned int &episode) {
  double none[1];
  return grid_allreduce<0>(gs, episode, none, nullptr);
}

// Streaming loads of read-only matrix data (never written by the kernel
// that reads them): non-coherent path, no L1 allocation.
__device__ __forceinline__ int ld_stream(const int *p) {
  int v;
  asm volatile("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_stream(const double *p) {
  double v;
  asm volatile("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ int16_t ld_stream16(const int16_t *p) {
  short v;
  asm volatile("ld.global.nc.L1::no_allocate.s16 %0, [%1];" : "=h"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float ld_stream(const float *p) {
  float v;
  asm volatile("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
// 16-byte and 8-byte streaming loads (p aligned to 16 / 8 bytes): one
// row's four FP32 weights, one row's four 16-bit column offsets.
__device__ __forceinline__ float4 ld_stream4(const float *p) {
  float4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p));
  return v;
}
__device__ __forceinline__ uint2 ld_stream_u2(const int16_t *p) {
  uint2 v;
  asm volatile("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];"
               : "=r"(v.x), "=r"(v.y)
               : "l"(p));
  return v;
}
// The k-th signed 16-bit offset of four packed in (lo, hi) words.
__device__ __forceinline__ int off16(uint2 v, int k) {
  const unsigned int w = (k < 2) ? v.x : v.y;
  return (int)(int16_t)(uint16_t)((k & 1) ? (w >> 16) : (w & 0xffffu));
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// y_row = (A x)_row for the lane's row of slice s, with x supplied by a
// functor (so callers can form x on the fly, e.g. p = z + beta*p).  Rows
// of width <= 4 (every cell of a triangle/quad mesh) issue all value and
// column loads before the gathers, so a warp has 8 independent streaming
// loads in flight per slice.
// Reference order: DIAG_FIRST  t = ad*x_i; t = t + a_k*x_k ...  (csrd)
//                  DIAG_LAST   t = a_1x_1 + ... + a_wx_w + ad*x_i (ellpack)
//                  DIAG_NONE   t = 0 + a_k*x_k ...                 (csr)
template <typename XF>
__device__ __forceinline__ double sell_row_f64(const SellView<double> &A, int s,
                                               int lane, int row, XF xf) {
  const int64_t base = A.sptr[s];
  int w = (int)((A.sptr[s + 1] - base) >> 5);
  FVC_CHK(w >= 0 && w <= A.n, A.chk, kChkSliceWidth, w = 0);
  const int *cp = A.col + base + lane;
  const double *vp = A.val + base + lane;
  double xd = 0.0;
  if (A.diag_mode != DIAG_NONE) xd = __dmul_rn(ld_stream(A.diag + row), xf(row));
  double t = (A.diag_mode == DIAG_FIRST) ? xd : 0.0;
  if (w <= 4) {
    int c[4];
    double a[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      c[k] = (k < w) ? ld_stream(cp + 32 * k) : 0;
      a[k] = (k < w) ? ld_stream(vp + 32 * k) : 0.0;
      FVC_CHK(k >= w || (unsigned)c[k] < (unsigned)A.n, A.chk, kChkColumn, c[k] = row);
    }
    if (A.diag_mode == DIAG_LAST) {
      // the reference's ELLPACK sums t1+t2+...+tw+t_diag left to right
      if (w > 0) t = __dmul_rn(a[0], xf(c[0]));
#pragma unroll
      for (int k = 1; k < 4; ++k)
        if (k < w) t = __dadd_rn(t, __dmul_rn(a[k], xf(c[k])));
      return __dadd_rn(t, xd);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < w) t = __dadd_rn(t, __dmul_rn(a[k], xf(c[k])));
    return t;
  }
  auto colk = [&](int k) {
    int c = ld_stream(cp + 32 * k);
    FVC_CHK((unsigned)c < (unsigned)A.n, A.chk, kChkColumn, c = row);
    return c;
  };
  if (A.diag_mode == DIAG_LAST) {
    t = __dmul_rn(ld_stream(vp), xf(colk(0)));
    for (int k = 1; k < w; ++k) t = __dadd_rn(t, __dmul_rn(ld_stream(vp + 32 * k), xf(colk(k))));
    return __dadd_rn(t, xd);
  }
  for (int k = 0; k < w; ++k) t = __dadd_rn(t, __dmul_rn(ld_stream(vp + 32 * k), xf(colk(k))));
  return t;
}

// The same row sum with fused multiply-adds (one FP64 instruction per
// term instead of two; GB300's FP64 pipe, ~1/64 of its FP32 rate, is the
// bottleneck of the FP64 solvers).  Terms are added in the same order.
template <typename XF>
__device__ __forceinline__ double sell_row_fma(const SellView<double> &A, int s, int lane,
                                               int row, XF xf) {
  const int64_t base = A.sptr[s];
  int w = (int)((A.sptr[s + 1] - base) >> 5);
  FVC_CHK(w >= 0 && w <= A.n, A.chk, kChkSliceWidth, w = 0);
  const int *cp = A.col + base + lane;
  const double *vp = A.val + base + lane;
  const bool has_diag = A.diag_mode != DIAG_NONE;
  const double dv = has_diag ? ld_stream(A.diag + row) : 0.0;
  const double xi = has_diag ? xf(row) : 0.0;
  double t = (A.diag_mode == DIAG_FIRST) ? dv * xi : 0.0;
  if (w <= 4) {
    int c[4];
    double a[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      c[k] = (k < w) ? ld_stream(cp + 32 * k) : 0;
      a[k] = (k < w) ? ld_stream(vp + 32 * k) : 0.0;
      FVC_CHK(k >= w || (unsigned)c[k] < (unsigned)A.n, A.chk, kChkColumn, c[k] = row);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < w) t = fma(a[k], xf(c[k]), t);
  } else {
    for (int k = 0; k < w; ++k) {
      int c = ld_stream(cp + 32 * k);
      FVC_CHK((unsigned)c < (unsigned)A.n, A.chk, kChkColumn, c = row);
      t = fma(ld_stream(vp + 32 * k), xf(c), t);
    }
  }
  if (A.diag_mode == DIAG_LAST) t = fma(dv, xi, t);
  return t;
}

// One system of a batch: its slices, its solver (1 PCG, 2 BiCGSTAB), its
// stopping tolerance, inner tolerance (mixed precision) and warm-start
// rule, its synchronisation state (counter, partials, nblocks and first
// block) and its result slots.
struct BatchSys {
  int s0, s1;
  int code, init;
  double tol, inner_tol;
  GridSync gs;
  double *result;
  int *iresult;
  // per-system mask (may be null: always solve).  *run == 0: the system is
  // not solved in this launch -- the reference's test before a solve
  // (the right-hand side's norm below 1e-32) skipped it -- and x keeps its
  // rows' values
  const int32_t *run = nullptr;
};

// A masked system's blocks leave at once; its lead block reports status
// FVC_OK after 0 iterations.  Every block of the group reads the same flag.
__device__ __forceinline__ bool batch_masked(const BatchSys &d, bool lead) {
  if (d.run == nullptr || *d.run != 0) return false;
  if (lead && threadIdx.x == 0) {
    d.iresult[0] = 0;
    d.iresult[1] = FVC_OK;
    d.iresult[2] = 0;
  }
  return true;
}

// y_row = (A^T x)_row over the stored matrix of a symmetric pattern: the
// entry (row, col(slot)) of A^T is the stored value of the mirror slot
// (col(slot), row); the diagonal is A's.  Terms in slot order, with FMA.
template <typename XF>
__device__ __forceinline__ double sell_row_fma_t(const SellView<double> &A, int s, int lane,
                                                 int row, XF xf) {
  const int64_t base = A.sptr[s];
  int w = (int)((A.sptr[s + 1] - base) >> 5);
  FVC_CHK(w >= 0 && w <= A.n, A.chk, kChkSliceWidth, w = 0);
  const int *cp = A.col + base + lane;
  const int *mp = A.mirror + base + lane;
  const bool has_diag = A.diag_mode != DIAG_NONE;
  const double dv = has_diag ? ld_stream(A.diag + row) : 0.0;
  double t = has_diag ? dv * xf(row) : 0.0;
#ifdef FVC_CHECK
  const int64_t nslots = A.sptr[A.nslices];
#endif
  if (w <= 4) {
    int c[4], m[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      c[k] = (k < w) ? ld_stream(cp + 32 * k) : 0;
      m[k] = (k < w) ? ld_stream(mp + 32 * k) : 0;
      FVC_CHK(k >= w || (unsigned)c[k] < (unsigned)A.n, A.chk, kChkColumn, c[k] = row);
      FVC_CHK(k >= w || (m[k] >= 0 && m[k] < nslots), A.chk, kChkMirror, m[k] = (int)(base + lane));
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < w) t = fma(A.val[m[k]], xf(c[k]), t);
  } else {
    for (int k = 0; k < w; ++k) {
      int c = ld_stream(cp + 32 * k), m = ld_stream(mp + 32 * k);
      FVC_CHK((unsigned)c < (unsigned)A.n, A.chk, kChkColumn, c = row);
      FVC_CHK(m >= 0 && m < nslots, A.chk, kChkMirror, m = (int)(base + lane));
      t = fma(A.val[m], xf(c), t);
    }
  }
  return t;
}

// A x (kT false) or A^T x (kT true) for one row
template <bool kT, typename XF>
__device__ __forceinline__ double row_fma(const SellView<double> &A, int s, int lane, int row,
                                          XF xf) {
  if (kT) return sell_row_fma_t(A, s, lane, row, xf);
  return sell_row_fma(A, s, lane, row, xf);
}

// Host side: scratch for the grid synchronisation of a persistent launch.
inline int32_t ensure_sync(Scratch &S, size_t nblocks) {
  const size_t need = 4 * kMaxNV * nblocks + 4 * kMaxNV;
  if (S.npart < need) {
    if (S.partials) cudaFree(S.partials);
    S.partials = nullptr;
    if (cudaMalloc(&S.partials, sizeof(double) * need) != cudaSuccess) return FVC_ERR_CUDA;
    S.npart = need;
  }
  if (!S.sync) {
    if (cudaMalloc(&S.sync, 64) != cudaSuccess) return FVC_ERR_CUDA;
    if (cudaMalloc(&S.err, 64) != cudaSuccess || cudaMemset(S.err, 0, 64) != cudaSuccess)
      return FVC_ERR_CUDA;
    if (cudaMalloc(&S.result, 16 * sizeof(double)) != cudaSuccess) return FVC_ERR_CUDA;
    if (cudaMalloc(&S.iresult, 16 * sizeof(int)) != cudaSuccess) return FVC_ERR_CUDA;
    if (cudaMalloc(&S.trace, 2 * kTraceMax * sizeof(double)) != cudaSuccess) return FVC_ERR_CUDA;
    if (cudaMalloc(&S.history, kHistoryMax * sizeof(float)) != cudaSuccess) return FVC_ERR_CUDA;
  }
  return FVC_OK;
}

inline GridSync make_sync(const Scratch &S, int nblocks) {
  GridSync g;
  g.count = S.sync;
  g.flag = S.sync + 8;  // separate 32-byte sector from the counter
  g.err = S.err;
  g.partials = S.partials;
  g.totals = S.partials + 4 * kMaxNV * (size_t)nblocks;
  g.nblocks = (unsigned int)nblocks;
  g.base = 0;
  return g;
}

// The word a failed device check records into (check builds): the second
// 32-byte sector of the launch's 64-byte error block, zeroed with it.  A
// separate word from the wait error, so that no wait gives up early (the
// staged kernels must see every bulk copy land); the launch runs to its end
// on the redirected indices and the host reads the word afterwards
// (check_word_status).
inline int *check_word(const Scratch &S) { return S.err ? S.err + 8 : nullptr; }
int32_t check_word_status(const Scratch &S, cudaStream_t stream);

inline void reset_sync(Scratch &S, cudaStream_t stream) {
  cudaMemsetAsync(S.sync, 0, 64, stream);
  cudaMemsetAsync(S.err, 0, 64, stream);
  cudaMemsetAsync(S.iresult, 0, 16 * sizeof(int), stream);
  cudaMemsetAsync(S.result, 0, 16 * sizeof(double), stream);
}

}  // namespace fvc
