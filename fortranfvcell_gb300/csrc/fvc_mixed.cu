// fvc_mixed.cu -- mixed-precision solves: FP32 Krylov inside an FP64
// defect-correction (iterative refinement) loop, one persistent launch.
//
//   outer sweep (FP64):  r = b - A x        (FP64 matrix, FP64 vectors)
//                        stop if ||r||2 <= refine_tol * ||b||2
//   inner solve (FP32):  S e = D^-1/2 r      S = D^-1/2 A D^-1/2, D = diag(A)
//                        CG (code 1) or BiCGSTAB (code 2), stopped after a
//                        relative reduction inner_tol of its own residual
//   update (FP64):       x = x + D^-1/2 e
//
// The symmetric Jacobi scaling is the reference's Jacobi preconditioner
// (m = ad, src/Solver.f:84) moved into the matrix, so the inner solver needs
// no preconditioner pass and S has a unit diagonal that is not stored.  It
// also keeps the 1e60 pressure pin of src/CellibPressure.f:557 inside the
// FP32 range (its row of S is O(1e-30) off the diagonal).  Dot products and
// norms accumulate in FP64.
#include <cmath>
#include <cstdio>

#include "fvc_device.cuh"
#include "fvc_internal.h"

namespace fvc {

namespace {

__global__ void scale_setup(int n, const double *__restrict__ jac, double *__restrict__ ds,
                            int *__restrict__ bad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    double m = jac[i];
    if (!(m > 0.0)) {
      atomicExch(bad, 1);
      ds[i] = 1.0;
    } else {
      ds[i] = 1.0 / sqrt(m);
    }
  }
}

__global__ void scale_values(int n, int nslices, const int64_t *__restrict__ sptr,
                             const int *__restrict__ col, const double *__restrict__ val,
                             const double *__restrict__ ds, float *__restrict__ val32) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += nw) {
    const int row = s * 32 + lane;
    const int64_t base = sptr[s];
    const int w = (int)((sptr[s + 1] - base) >> 5);
    const double dr = (row < n) ? ds[row] : 0.0;
    for (int k = 0; k < w; ++k) {
      int64_t q = base + 32 * k + lane;
      val32[q] = (row < n) ? (float)(val[q] * dr * ds[col[q]]) : 0.0f;
    }
  }
}

struct MArgs {
  SellView<double> A;   // FP64 matrix (residuals)
  const float *val32;   // S values (same slots as A)
  int unit_diag;        // 1: S has an implicit unit diagonal
  const double *ds;     // D^-1/2
  const double *b;
  double *x;
  double *rd;           // FP64 residual scratch (unused slot reserved)
  float *rs, *pa, *pb, *q, *e, *r0, *v, *t;
  double *partials;
  GridSync gs;
  double target;        // refine tolerance on ||b-Ax||/||b||
  double inner_tol;
  int max_refine;
  int maxit;            // cap on total inner iterations
  int init;
  double *result;
  int *iresult;
};

constexpr int kNV = 4;

__device__ __forceinline__ double *mslot(const MArgs &a, int rot, int q) {
  return a.partials + ((size_t)(rot & 3) * kNV + q) * gridDim.x;
}

template <int NV>
__device__ __forceinline__ bool mreduce(const MArgs &a, int &rot, double (&v)[NV], double *red,
                                        double *tot) {
  block_sum<NV>(v, red);
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < NV; ++q) mslot(a, rot, q)[blockIdx.x] = v[q];
  if (!grid_barrier(a.gs)) return false;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp < NV) {
    const double *p = mslot(a, rot, warp);
    double t = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) t += __ldcg(p + b);
    t = warp_sum(t);
    if (lane == 0) tot[warp] = t;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = tot[q];
  __syncthreads();
  ++rot;
  return true;
}

// (S y)_row with y supplied by a functor, FP32 arithmetic.
template <typename YF>
__device__ __forceinline__ float srow(const MArgs &a, int s, int lane, int row, YF yf) {
  const int64_t base = a.A.sptr[s];
  const int w = (int)((a.A.sptr[s + 1] - base) >> 5);
  float t = a.unit_diag ? yf(row) : 0.0f;
  const int *cp = a.A.col + base + lane;
  const float *vp = a.val32 + base + lane;
#pragma unroll 4
  for (int k = 0; k < w; ++k) t = fmaf(ld_stream(vp + 32 * k), yf(ld_stream(cp + 32 * k)), t);
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

// FP64 residual sweep: rs = D^-1/2 (b - A x) in FP32, returns ||b-Ax||^2,
// ||b||^2 and ||rs||^2.
__device__ __forceinline__ bool residual_sweep(const MArgs &a, int &rot, bool zero_x,
                                               double (&out)[3], double *red, double *tot) {
  const MPart P(a.A.nslices, a.A.n);
  double acc[3] = {0.0, 0.0, 0.0};
  const double *x = a.x;
  MFOR_ROWS(P) {
    double ax = zero_x ? 0.0 : sell_row_f64(a.A, s_, P.lane, row, [&](int k) { return x[k]; });
    if (zero_x) a.x[row] = 0.0;
    double bi = a.b[row];
    double ri = bi - ax;
    float rsi = (float)(a.ds[row] * ri);
    a.rs[row] = rsi;
    acc[0] += ri * ri;
    acc[1] += bi * bi;
    acc[2] += (double)rsi * (double)rsi;
  }
  if (!mreduce<3>(a, rot, acc, red, tot)) return false;
  out[0] = acc[0];
  out[1] = acc[1];
  out[2] = acc[2];
  return true;
}

// x += D^-1/2 e (FP64), own rows; caller places a barrier after it.
__device__ __forceinline__ void apply_correction(const MArgs &a) {
  const MPart P(a.A.nslices, a.A.n);
  MFOR_ROWS(P) { a.x[row] = a.x[row] + a.ds[row] * (double)a.e[row]; }
}

__global__ void __launch_bounds__(256) mixed_cg(MArgs a) {
  __shared__ double red[kNV * 32];
  __shared__ double tot[kNV];
  const MPart P(a.A.nslices, a.A.n);
  int rot = 0, sweep = 0, inner_total = 0, status = FVC_ERR_NOCONV;
  double res[3];
  double relres = 0.0, bnorm2 = 0.0;
  bool zero_x = a.init != 0;
  for (sweep = 0; sweep <= a.max_refine; ++sweep) {
    if (!residual_sweep(a, rot, zero_x, res, red, tot)) return;
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
    // inner CG on S e = rs from e = 0
    double rz = res[2];
    const double stop2 = a.inner_tol * a.inner_tol * rz;
    float beta = 0.0f;
    float *pprev = a.rs, *pcur = a.pa;
    int it = 0;
    for (;;) {
      ++it;
      double acc[1] = {0.0};
      const float *pp = pprev;
      const float *rr = a.rs;
      if (it == 1) {
        MFOR_ROWS(P) {
          float qi = srow(a, s_, P.lane, row, [&](int k) { return rr[k]; });
          float pi = rr[row];
          pcur[row] = pi;
          a.e[row] = 0.0f;
          a.q[row] = qi;
          acc[0] += (double)pi * (double)qi;
        }
      } else {
        MFOR_ROWS(P) {
          auto pf = [&](int k) { return fmaf(beta, pp[k], rr[k]); };
          float pi = pf(row);
          pcur[row] = pi;
          float qi = srow(a, s_, P.lane, row, pf);
          a.q[row] = qi;
          acc[0] += (double)pi * (double)qi;
        }
      }
      if (!mreduce<1>(a, rot, acc, red, tot)) return;
      const float alpha = (float)(rz / acc[0]);
      acc[0] = 0.0;
      MFOR_ROWS(P) {
        float pi = pcur[row];
        a.e[row] = fmaf(alpha, pi, a.e[row]);
        float ri = fmaf(-alpha, a.q[row], a.rs[row]);
        a.rs[row] = ri;
        acc[0] += (double)ri * (double)ri;
      }
      if (!mreduce<1>(a, rot, acc, red, tot)) return;
      const double rz_new = acc[0];
      beta = (float)(rz_new / rz);
      rz = rz_new;
      if (!(rz == rz)) break;
      if (rz <= stop2 || inner_total + it >= a.maxit) break;
      pprev = pcur;
      pcur = (pcur == a.pa) ? a.pb : a.pa;
    }
    inner_total += it;
    apply_correction(a);
    if (!grid_barrier(a.gs)) return;
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

// BiCGSTAB inner solver (unpreconditioned, on S).
__global__ void __launch_bounds__(256) mixed_bicgstab(MArgs a) {
  __shared__ double red[kNV * 32];
  __shared__ double tot[kNV];
  const MPart P(a.A.nslices, a.A.n);
  int rot = 0, sweep = 0, inner_total = 0, status = FVC_ERR_NOCONV;
  double res[3];
  double relres = 0.0, bnorm2 = 0.0;
  bool zero_x = a.init != 0;
  float *sv = a.rs, *p = a.pa, *v = a.q, *t = a.t, *r0 = a.r0, *e = a.e;
  for (sweep = 0; sweep <= a.max_refine; ++sweep) {
    if (!residual_sweep(a, rot, zero_x, res, red, tot)) return;
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
    double rho = res[2];
    const double stop2 = a.inner_tol * a.inner_tol * res[2];
    MFOR_ROWS(P) {
      float si = sv[row];
      r0[row] = si;
      p[row] = si;
      e[row] = 0.0f;
    }
    if (!grid_barrier(a.gs)) return;
    int it = 0;
    for (;;) {
      ++it;
      double acc1[1] = {0.0};
      MFOR_ROWS(P) {
        float vi = srow(a, s_, P.lane, row, [&](int k) { return p[k]; });
        v[row] = vi;
        acc1[0] += (double)r0[row] * (double)vi;
      }
      if (!mreduce<1>(a, rot, acc1, red, tot)) return;
      const float alpha = (float)(rho / acc1[0]);
      double acc[2];
      MFOR_ROWS(P) { sv[row] = fmaf(-alpha, v[row], sv[row]); }
      if (!grid_barrier(a.gs)) return;
      acc[0] = acc[1] = 0.0;
      MFOR_ROWS(P) {
        float ti = srow(a, s_, P.lane, row, [&](int k) { return sv[k]; });
        t[row] = ti;
        acc[0] += (double)ti * (double)sv[row];
        acc[1] += (double)ti * (double)ti;
      }
      if (!mreduce<2>(a, rot, acc, red, tot)) return;
      const float omega = (acc[1] > 0.0) ? (float)(acc[0] / acc[1]) : 0.0f;
      double acc2[2] = {0.0, 0.0};
      MFOR_ROWS(P) {
        float si = sv[row];
        e[row] = fmaf(omega, si, fmaf(alpha, p[row], e[row]));
        float sn = fmaf(-omega, t[row], si);
        sv[row] = sn;
        acc2[0] += (double)r0[row] * (double)sn;
        acc2[1] += (double)sn * (double)sn;
      }
      if (!mreduce<2>(a, rot, acc2, red, tot)) return;
      const double rho_new = acc2[0];
      if (!(acc2[1] == acc2[1]) || acc2[1] <= stop2 || inner_total + it >= a.maxit || omega == 0.0f ||
          rho_new == 0.0)
        break;
      const float beta = (float)((rho_new / rho) * ((double)alpha / (double)omega));
      rho = rho_new;
      MFOR_ROWS(P) { p[row] = fmaf(beta, fmaf(-omega, v[row], p[row]), sv[row]); }
      if (!grid_barrier(a.gs)) return;
    }
    inner_total += it;
    apply_correction(a);
    if (!grid_barrier(a.gs)) return;
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
  if (!A.val32 && cudaMalloc(&A.val32, sizeof(float) * (size_t)std::max<int64_t>(A.slots, 1)) != cudaSuccess)
    return FVC_ERR_CUDA;
  if (!A.dscale && cudaMalloc(&A.dscale, sizeof(double) * (size_t)A.n) != cudaSuccess)
    return FVC_ERR_CUDA;
  int *bad = nullptr;
  if (cudaMalloc(&bad, sizeof(int)) != cudaSuccess) return FVC_ERR_CUDA;
  cudaMemsetAsync(bad, 0, sizeof(int), stream);
  scale_setup<<<(A.n + 255) / 256, 256, 0, stream>>>(A.n, A.jac, A.dscale, bad);
  count_launch();
  int blocks = std::max(1, std::min((A.nslices + 7) / 8, sm_count_m() * 8));
  scale_values<<<blocks, 256, 0, stream>>>(A.n, A.nslices, A.sptr, A.col, A.val, A.dscale, A.val32);
  count_launch();
  int hbad = 0;
  cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, stream);
  cudaError_t ce = cudaStreamSynchronize(stream);
  cudaFree(bad);
  if (ce != cudaSuccess) return FVC_ERR_CUDA;
  if (hbad) return FVC_ERR_UNSUPPORTED;  // Jacobi scaling needs ad > 0
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
    for (int i = 0; i < 8; ++i) {
      if (S.f[i]) cudaFree(S.f[i]);
      S.f[i] = nullptr;
    }
    S.nf = n;
  }
  for (int i = 0; i < 8; ++i)
    if (!S.f[i] && cudaMalloc(&S.f[i], sizeof(float) * (n + 64)) != cudaSuccess) return FVC_ERR_CUDA;
  auto kern = (code == 1) ? mixed_cg : mixed_bicgstab;
  const int threads = (o.block_threads > 0) ? o.block_threads : 256;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, 0);
  if (occ <= 0) occ = 1;
  if (o.blocks_per_sm > 0 && o.blocks_per_sm < occ) occ = o.blocks_per_sm;
  const int warps = threads / 32;
  int blocks = std::max(1, std::min(occ * sm_count_m(), (A.nslices + warps - 1) / warps));
  size_t need = 4 * kNV * (size_t)blocks;
  if (S.npart < need) {
    if (S.partials) cudaFree(S.partials);
    if (cudaMalloc(&S.partials, sizeof(double) * need) != cudaSuccess) return FVC_ERR_CUDA;
    S.npart = need;
  }
  if (!S.sync) {
    if (cudaMalloc(&S.sync, 64) != cudaSuccess) return FVC_ERR_CUDA;
    if (cudaMalloc(&S.err, 64) != cudaSuccess) return FVC_ERR_CUDA;
    if (cudaMalloc(&S.result, 16 * sizeof(double)) != cudaSuccess) return FVC_ERR_CUDA;
    if (cudaMalloc(&S.iresult, 16 * sizeof(int)) != cudaSuccess) return FVC_ERR_CUDA;
  }
  cudaMemsetAsync(S.sync, 0, 64, stream);
  cudaMemsetAsync(S.err, 0, 64, stream);
  cudaMemsetAsync(S.iresult, 0, 16 * sizeof(int), stream);
  cudaMemsetAsync(S.result, 0, 16 * sizeof(double), stream);
  MArgs a{};
  a.A.n = A.n;
  a.A.nslices = A.nslices;
  a.A.sptr = A.sptr;
  a.A.col = A.col;
  a.A.val = A.val;
  a.A.diag = A.diag;
  a.A.diag_mode = A.diag_mode;
  a.val32 = A.val32;
  a.unit_diag = (A.diag_mode != DIAG_NONE) ? 1 : 0;
  a.ds = A.dscale;
  a.b = b;
  a.x = x;
  a.rs = S.f[0];
  a.pa = S.f[1];
  a.pb = S.f[2];
  a.q = S.f[3];
  a.e = S.f[4];
  a.r0 = S.f[5];
  a.t = S.f[6];
  a.v = S.f[7];
  a.partials = S.partials;
  a.gs.count = S.sync;
  a.gs.gen = S.sync + 1;
  a.gs.err = S.err;
  a.gs.nblocks = (unsigned)blocks;
  a.target = (o.refine_tol > 0) ? o.refine_tol : tol;
  a.inner_tol = (o.inner_tol > 0) ? o.inner_tol : 1e-4;
  a.max_refine = (o.max_refine > 0) ? o.max_refine : 30;
  a.maxit = maxit;
  a.init = init;
  a.result = S.result;
  a.iresult = S.iresult;
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
    st->refinements = ires[0];
    st->energy = 0.0;
    st->conv = a.target;
    st->final_crit = res[2];
    st->rel_residual = res[2];
    st->solve_ms = ms;
  }
  return ires[1];
}

}  // namespace fvc
