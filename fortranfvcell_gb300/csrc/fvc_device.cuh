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
};

// Scalars of one solve that every block computes identically from the
// same reduction partials.
struct GridSync {
  unsigned int *count;   // arrival counter
  unsigned int *gen;     // generation
  int *err;              // sticky error (FVC_ERR_TIMEOUT on a stuck wait)
  unsigned int nblocks;
};

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier for a cooperative (co-resident) launch.  The wait is
// bounded: after kBarrierTimeoutNs the block records FVC_ERR_TIMEOUT and
// leaves; every other waiter sees the flag and leaves too, so a broken
// launch returns an error instead of spinning.  Returns false on error.
constexpr uint64_t kBarrierTimeoutNs = 4000000000ull;  // 4 s

__device__ __forceinline__ bool grid_barrier(const GridSync &gs) {
  __syncthreads();
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    volatile unsigned int *vgen = gs.gen;
    volatile int *verr = gs.err;
    unsigned int my_gen = *vgen;
    __threadfence();
    unsigned int arrived = atomicAdd(gs.count, 1u);
    if (arrived == gs.nblocks - 1) {
      *gs.count = 0;
      __threadfence();
      atomicAdd(gs.gen, 1u);
    } else {
      uint64_t t0 = global_ns();
      unsigned int spins = 0;
      while (*vgen == my_gen) {
        if (*verr != 0) break;
        if ((++spins & 63u) == 0 && global_ns() - t0 > kBarrierTimeoutNs) {
          atomicExch(gs.err, 7 /* FVC_ERR_TIMEOUT */);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = (*verr == 0);
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
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

// Sum of the per-block partials of NV reductions, read after a barrier.
// Every block runs the same fixed-order sum, so all blocks obtain the
// same bits without a broadcast.  Result valid in all threads.
template <int NV>
__device__ __forceinline__ void grid_total(const double *partials, int nblocks,
                                           double (&out)[NV], double *sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp < NV) {
    const double *p = partials + (size_t)warp * nblocks;
    double t = 0.0;
    for (int b = lane; b < nblocks; b += 32) t = __dadd_rn(t, __ldcg(p + b));
    t = warp_sum(t);
    if (lane == 0) sh[warp] = t;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) out[q] = sh[q];
  __syncthreads();
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
__device__ __forceinline__ float ld_stream(const float *p) {
  float v;
  asm volatile("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}

// y_row = (A x)_row for the lane's row of slice s, with x supplied by a
// functor (so callers can form x on the fly, e.g. p = z + beta*p).
// Reference order: DIAG_FIRST  t = ad*x_i; t = t + a_k*x_k ...  (csrd)
//                  DIAG_LAST   t = a_1x_1 + ... + a_wx_w + ad*x_i (ellpack)
//                  DIAG_NONE   t = 0 + a_k*x_k ...                 (csr)
template <typename XF>
__device__ __forceinline__ double sell_row_f64(const SellView<double> &A, int s,
                                               int lane, int row, XF xf) {
  const int64_t base = A.sptr[s];
  const int w = (int)((A.sptr[s + 1] - base) >> 5);
  double t;
  double xd = 0.0;
  if (A.diag_mode != DIAG_NONE) xd = __dmul_rn(ld_stream(A.diag + row), xf(row));
  if (A.diag_mode == DIAG_FIRST) {
    t = xd;
  } else {
    t = 0.0;
  }
  const int *cp = A.col + base + lane;
  const double *vp = A.val + base + lane;
  if (A.diag_mode == DIAG_LAST) {
    // the reference's ELLPACK sums t1+t2+...+tw+t_diag left to right
    if (w > 0) t = __dmul_rn(ld_stream(vp), xf(ld_stream(cp)));
    for (int k = 1; k < w; ++k)
      t = __dadd_rn(t, __dmul_rn(ld_stream(vp + 32 * k), xf(ld_stream(cp + 32 * k))));
    t = __dadd_rn(t, xd);
  } else {
    for (int k = 0; k < w; ++k)
      t = __dadd_rn(t, __dmul_rn(ld_stream(vp + 32 * k), xf(ld_stream(cp + 32 * k))));
  }
  return t;
}

}  // namespace fvc
