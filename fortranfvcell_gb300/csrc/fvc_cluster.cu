// fvc_cluster.cu -- Jacobi-PCG (src/Iterativos.f:29-106) of a small system
// on one thread-block cluster, resident in distributed shared memory.
//
// A system of a few thousand rows (the SIMPLE p' system of a 64 x 64 cavity
// has 4096) leaves a grid-wide persistent kernel latency-bound: every
// iteration waits twice for all blocks through L2 atomics and reads its
// vectors from L2.  Here the rows are split over the CTAs of one cluster
// (up to 16 SMs).  Each CTA copies its rows' SELL slices, diagonal and
// Jacobi weights into shared memory once and keeps x, r, z, p and q there;
// the SpMV reads a neighbour row's p from the owning CTA's shared memory
// over DSMEM, and each reduction is one cluster barrier: every CTA posts its
// partial in its own shared memory, and after the barrier every CTA sums
// all partials in rank order itself (identical totals in every CTA, so
// every CTA takes the same branch).  Per iteration: form p, barrier, SpMV +
// p.q, reduction, update + r.z, reduction -- three cluster barriers and no
// global-memory traffic.
//
// There is no spin-wait: the only waits are hardware cluster barriers, which
// every CTA reaches the same number of times (the loop exit depends only on
// the identical totals and maxit), and a last barrier keeps every CTA's
// shared memory alive until the others have finished reading it.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "fvc_device.cuh"
#include "fvc_internal.h"

namespace cg = cooperative_groups;

namespace fvc {
namespace {

constexpr int kClMax = 16;        // CTAs per cluster (non-portable above 8)
constexpr int kClMaxRows = 2048;  // rows per CTA
// Largest system run on a cluster: measured per PCG iteration on GB300 (16
// CTAs, 256 rows each) against the grid-wide kernel: 4096 rows 6.65 vs
// 8.41 us, 6124 rows 7.59 vs 8.41 us, 10000 rows 9.59 vs 8.95 us.  Forming
// p at every read instead of the p barrier was slower at every size.  The
// FP64 rate of the cluster's SMs bounds it: 512 or 1024 rows per CTA
// instead of 256 (8 or 4 CTAs for 4096 rows) took a 64^2 cavity's 200
// outer iterations from 0.67 s to 0.81 and 1.13 s.
constexpr int kClMaxN = 8192;

struct ClArgs {
  SellView<double> A;
  const double *minv, *b;
  double *x;
  int R;            // rows per CTA, a multiple of 32
  double tol;
  int maxit, init, stop_rule;
  double *result;   // [0] energy [1] conv [2] final_crit [3] |b-Ax|^2 [4] |b|^2
  int *iresult;     // [0] iterations [1] status
};

// shared-memory layout of one CTA (R rows, S slots)
struct ClLayout {
  int R, S;
  __host__ __device__ size_t bytes() const {
    return (size_t)7 * R * sizeof(double) + (size_t)S * (sizeof(double) + sizeof(int)) +
           (size_t)(R / 32 + 1) * sizeof(int);
  }
};

extern __shared__ __align__(16) unsigned char cl_smem[];

template <int NV, typename F>
__device__ __forceinline__ void cluster_allreduce(cg::cluster_group &cl, unsigned int &ep,
                                                  double (&v)[NV], double (*part)[kMaxNV],
                                                  double *red, F &&f) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const double t = warp_sum(v[q]);
    if (lane == 0) red[q * 32 + warp] = t;
  }
  __syncthreads();
  const unsigned int slot = ep++ & 1u;  // two slots: a CTA one reduction ahead never
                                       // overwrites a partial still being read
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const double t = warp_sum(lane < nwarps ? red[q * 32 + lane] : 0.0);
      if (lane == 0) part[slot][q] = t;
    }
  }
  cl.sync();
  if (warp == 0) {
    const int nb = (int)cl.num_blocks();
    double t[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double u = 0.0;
      if (lane < nb) u = *cl.map_shared_rank(&part[slot][q], lane);
      t[q] = warp_sum(u);
    }
    if (lane == 0) f(t);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(1024) pcg_cluster(ClArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  __shared__ double red[kMaxNV * 32];
  __shared__ double part[2][kMaxNV];
  __shared__ double *rp[kClMax];  // each CTA's p, mapped into the cluster window
  __shared__ double *rx[kClMax];  // and its x
  __shared__ struct {
    double d, alpha, beta, conv, crit;
    int stop;
  } sh;
  const int rank = (int)cl.block_rank(), nb = (int)cl.num_blocks();
  const int R = a.R, n = a.A.n;
  const int r0 = rank * R;
  const int rows = max(0, min(R, n - r0));
  const int ns = (rows + 31) / 32, s0 = r0 / 32;
  const int64_t sbase = a.A.sptr[s0];
  const int S = (int)(a.A.sptr[s0 + ns] - sbase);
  double *p = reinterpret_cast<double *>(cl_smem);
  double *x = p + R, *r = x + R, *z = r + R, *q = z + R, *mi = q + R, *dg = mi + R;
  double *val = dg + R;
  int *col = reinterpret_cast<int *>(val + S);  // (owner << 16) | local row
  int *sp = col + S;                            // slot offset of each local slice
  const bool has_diag = a.A.diag_mode != DIAG_NONE;
#ifdef FVC_CHECK
  // check builds: columns outside [0, n) (whose owner CTA would not be in
  // the cluster) are counted here, redirected to this CTA's first row, and
  // end the solve uniformly after the first reduction
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
#endif
  // load the rows' slices (columns re-coded as owner CTA and local row)
  for (int i = threadIdx.x; i <= ns; i += blockDim.x) sp[i] = (int)(a.A.sptr[s0 + i] - sbase);
  for (int k = threadIdx.x; k < S; k += blockDim.x) {
    int c = a.A.col[sbase + k];
    FVC_CHK((unsigned)c < (unsigned)n, &s_bad, kChkCluster, c = r0);
    const int owner = c / R;
    col[k] = (owner << 16) | (c - owner * R);
    val[k] = a.A.val[sbase + k];
  }
  for (int i = threadIdx.x; i < R; i += blockDim.x) {
    const bool own = i < rows;
    mi[i] = own ? a.minv[r0 + i] : 0.0;
    dg[i] = (own && has_diag) ? a.A.diag[r0 + i] : 0.0;
    x[i] = (own && !a.init) ? a.x[r0 + i] : 0.0;
    p[i] = 0.0;
  }
  if (threadIdx.x < nb) {
    rp[threadIdx.x] = cl.map_shared_rank(p, (int)threadIdx.x);
    rx[threadIdx.x] = cl.map_shared_rank(x, (int)threadIdx.x);
  }
  cl.sync();  // every CTA's x and maps in place

  // y_i = (A v)_i over the local row i with the reference's diagonal order;
  // xf(owner, local) reads v
  auto spmv_row = [&](int i, auto xf) -> double {
    const int sl = i >> 5, lane = i & 31;
    const int base = sp[sl], w = (sp[sl + 1] - base) >> 5;
    const double xi = xf(rank, i);
    double t = (a.A.diag_mode == DIAG_FIRST) ? dg[i] * xi : 0.0;
    if (w <= 4) {
      int c[4];
      double v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        c[k] = (k < w) ? col[base + 32 * k + lane] : 0;
        v[k] = (k < w) ? val[base + 32 * k + lane] : 0.0;
      }
      double xv[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) xv[k] = (k < w) ? xf(c[k] >> 16, c[k] & 0xffff) : 0.0;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k < w) t = fma(v[k], xv[k], t);
    } else {
      for (int k = 0; k < w; ++k) {
        const int c = col[base + 32 * k + lane];
        t = fma(val[base + 32 * k + lane], xf(c >> 16, c & 0xffff), t);
      }
    }
    if (a.A.diag_mode == DIAG_LAST) t = fma(dg[i], xi, t);
    return t;
  };
  auto xread = [&](int o, int l) { return (o == rank) ? x[l] : rx[o][l]; };

  unsigned int ep = 0;
  const bool rule0 = a.stop_rule == 0;
  // r = b - A x ; z = r/m ; p = z ; d = r.z
#ifdef FVC_CHECK
  double acc[3] = {0.0, 0.0, (threadIdx.x == 0 && s_bad != 0) ? 1.0 : 0.0};
#else
  double acc[2] = {0.0, 0.0};
#endif
  for (int i = threadIdx.x; i < rows; i += blockDim.x) {
    const double ax = a.init ? 0.0 : spmv_row(i, xread);
    const double bi = a.b[r0 + i];
    const double ri = bi - ax;
    const double zi = ri * mi[i];
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
    acc[0] = fma(ri, zi, acc[0]);
    acc[1] = fma(bi, bi, acc[1]);
  }
#ifdef FVC_CHECK
  cluster_allreduce<3>(cl, ep, acc, part, red, [&](const double *t) {
    sh.stop = (t[2] > 0.0) ? 3 : 0;
#else
  cluster_allreduce<2>(cl, ep, acc, part, red, [&](const double *t) {
    sh.stop = 0;
#endif
    sh.d = t[0];
    sh.conv = rule0 ? a.tol * sqrt(fabs(t[0])) : a.tol * sqrt(t[1]);
    sh.crit = 0.0;
  });
  int j, status = FVC_OK;
  double beta = 0.0;
  const int jmax = (sh.stop == 3) ? 0 : a.maxit;  // 3: a failed check (check builds)
  if (sh.stop == 3) status = FVC_ERR_ARG;
  for (j = 1; j <= jmax; ++j) {
    if (j > 1) {  // p = z + beta p on the own rows, then visible to the cluster
      for (int i = threadIdx.x; i < rows; i += blockDim.x) p[i] = fma(beta, p[i], z[i]);
      cl.sync();
    }
    double pq[1] = {0.0};
    for (int i = threadIdx.x; i < rows; i += blockDim.x) {
      const double qi = spmv_row(i, [&](int o, int l) { return (o == rank) ? p[l] : rp[o][l]; });
      q[i] = qi;
      pq[0] = fma(p[i], qi, pq[0]);
    }
    cluster_allreduce<1>(cl, ep, pq, part, red, [&](const double *t) { sh.alpha = sh.d / t[0]; });
    const double alpha = sh.alpha;
    double rz[2] = {0.0, 0.0};
    for (int i = threadIdx.x; i < rows; i += blockDim.x) {
      x[i] = fma(alpha, p[i], x[i]);
      const double ri = fma(-alpha, q[i], r[i]);
      const double zi = ri * mi[i];
      r[i] = ri;
      z[i] = zi;
      rz[0] = fma(ri, zi, rz[0]);
      rz[1] = fma(ri, ri, rz[1]);
    }
    cluster_allreduce<2>(cl, ep, rz, part, red, [&](const double *t) {
      sh.beta = t[0] / sh.d;
      sh.d = sh.beta * sh.d;
      sh.crit = rule0 ? sqrt(fabs(sh.d)) : sqrt(t[1]);
      sh.stop = (!(sh.crit == sh.crit) || isinf(sh.d)) ? 2 : (sh.crit < sh.conv ? 1 : 0);
    });
    if (sh.stop == 2) {
      status = FVC_ERR_NAN;
      break;
    }
    if (sh.stop == 1) break;
    beta = sh.beta;
  }
  if (j > a.maxit && status == FVC_OK) {
    j = a.maxit;
    status = FVC_ERR_NOCONV;
  }
  if (status == FVC_ERR_ARG) j = 0;
  // x.Ax, |b - Ax|^2, |b|^2 (x complete in every CTA after the barrier)
  cl.sync();
  double e3[3] = {0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < rows; i += blockDim.x) {
    const double ax = spmv_row(i, xread);
    const double bi = a.b[r0 + i], rr = bi - ax;
    e3[0] = fma(x[i], ax, e3[0]);
    e3[1] = fma(rr, rr, e3[1]);
    e3[2] = fma(bi, bi, e3[2]);
    a.x[r0 + i] = x[i];
  }
  cluster_allreduce<3>(cl, ep, e3, part, red, [&](const double *t) {
    if (rank == 0) {
      a.result[0] = t[0];
      a.result[1] = sh.conv;
      a.result[2] = sh.crit;
      a.result[3] = t[1];
      a.result[4] = t[2];
      a.iresult[0] = j;
      a.iresult[1] = status;
      a.iresult[2] = 0;
    }
  });
  cl.sync();  // no CTA leaves while another may still read its shared memory
}

// The cluster layout of an n-row system: CTAs, rows per CTA (a multiple of
// 32, at most kClMaxRows, over at most kClMax CTAs).  False when the system
// does not fit one cluster.
bool cluster_shape(int n, int &nb, int &R) {
  if (n <= 0 || n > kClMaxN) return false;
  nb = std::min(kClMax, std::max(1, (n + 255) / 256));
  R = ((n + nb - 1) / nb + 31) / 32 * 32;
  if (R > kClMaxRows) return false;
  nb = (n + R - 1) / R;
  return true;
}

}  // namespace

// Largest number of stored slots of one CTA's rows under the cluster
// layout, from the host copy of the slice pointers; -1 when the system does
// not fit one cluster.
int cluster_slots_max(int n, int nslices, const int64_t *sptr) {
  int nb = 0, R = 0;
  if (!sptr || !cluster_shape(n, nb, R)) return -1;
  int smax = 0;
  for (int c = 0; c < nb; ++c) {
    const int s0 = c * R / 32, s1 = std::min(nslices, (c + 1) * R / 32);
    smax = std::max(smax, (int)(sptr[s1] - sptr[s0]));
  }
  return smax;
}

// Enqueues the cluster PCG when the system fits one cluster and returns
// without waiting; FVC_ERR_UNSUPPORTED (and nothing enqueued) when it does
// not, so the caller falls back to the grid-wide kernel.  launch = false
// only checks the fit and prepares the scratch.
int32_t enqueue_pcg_cluster(const DeviceMatrix &A, Scratch &S, const double *b, double *x,
                            double tol, int maxit, int init, const fvc_opts &o,
                            cudaStream_t stream, bool launch) {
  const int n = A.n;
  if (n <= 0 || A.diag_mode == DIAG_NONE || !A.jinv) return FVC_ERR_UNSUPPORTED;
  int nb = 0, R = 0;
  if (!cluster_shape(n, nb, R)) return FVC_ERR_UNSUPPORTED;
  int smax = A.cl_smax;
  if (smax < 0) {  // a matrix loaded without the host-side count
    std::vector<int64_t> sptr((size_t)A.nslices + 1);
    if (cudaMemcpyAsync(sptr.data(), A.sptr, sizeof(int64_t) * sptr.size(),
                        cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess)
      return FVC_ERR_CUDA;
    smax = cluster_slots_max(n, A.nslices, sptr.data());
  }
  const ClLayout L{R, smax};
  const size_t smem = L.bytes();
  if (smem > 200 * 1024) return FVC_ERR_UNSUPPORTED;
  static bool attrs_set = false;
  if (!attrs_set) {
    cudaFuncSetAttribute(pcg_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(pcg_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    attrs_set = true;
  }
  const int threads = std::min(1024, std::max(128, (R + 127) / 128 * 128));
  if (ensure_sync(S, 1) != FVC_OK) return FVC_ERR_CUDA;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)nb);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)nb;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, pcg_cluster, &cfg) != cudaSuccess ||
      clusters < 1) {
    cudaGetLastError();
    return FVC_ERR_UNSUPPORTED;
  }
  if (!launch) return FVC_OK;
  cudaMemsetAsync(S.err, 0, 64, stream);  // the whole error block (wait and check words)
  cudaMemsetAsync(S.iresult, 0, 16 * sizeof(int), stream);
  cudaMemsetAsync(S.result, 0, 16 * sizeof(double), stream);
  ClArgs a{};
  a.A = SellView<double>{A.n, A.nslices, A.sptr, A.col, A.val, A.diag, A.diag_mode};
  a.minv = A.jinv;
  a.b = b;
  a.x = x;
  a.R = R;
  a.tol = tol;
  a.maxit = maxit;
  a.init = init;
  a.stop_rule = o.stop_rule;
  a.result = S.result;
  a.iresult = S.iresult;
  const cudaError_t ce = cudaLaunchKernelEx(&cfg, pcg_cluster, a);
  count_launch();
  if (ce != cudaSuccess) {
    fprintf(stderr, "fvcgpu: cluster PCG launch failed: %s\n", cudaGetErrorString(ce));
    cudaGetLastError();
    return FVC_ERR_CUDA;
  }
  return FVC_OK;
}

// Runs the cluster PCG synchronously (FVC_ERR_UNSUPPORTED when the system
// does not fit one cluster).
int32_t run_pcg_cluster(const DeviceMatrix &A, Scratch &S, const double *b, double *x,
                        double tol, int maxit, int init, const fvc_opts &o, cudaStream_t stream,
                        fvc_stats *st) {
  int32_t rc = enqueue_pcg_cluster(A, S, b, x, tol, maxit, init, o, stream, false);
  if (rc != FVC_OK) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, stream);
  rc = enqueue_pcg_cluster(A, S, b, x, tol, maxit, init, o, stream, true);
  cudaEventRecord(e1, stream);
  if (rc != FVC_OK) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  double res[16];
  int ires[16];
  cudaMemcpyAsync(res, S.result, sizeof(res), cudaMemcpyDeviceToHost, stream);
  cudaMemcpyAsync(ires, S.iresult, sizeof(ires), cudaMemcpyDeviceToHost, stream);
  const cudaError_t ce = cudaStreamSynchronize(stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ce != cudaSuccess) {
    fprintf(stderr, "fvcgpu: cluster PCG failed: %s\n", cudaGetErrorString(ce));
    return FVC_ERR_CUDA;
  }
#ifdef FVC_CHECK
  if (ires[1] == FVC_ERR_ARG)
    fprintf(stderr, "fvcgpu: device check failed: cluster PCG column outside [0, n) (code %d); "
                    "the solve's result is void\n", (int)kChkCluster);
#endif
  if (st) {
    st->status = ires[1];
    st->iterations = ires[0];
    st->inner_iterations = 0;
    st->refinements = 0;
    st->energy = res[0];
    st->conv = res[1];
    st->final_crit = res[2];
    st->rel_residual = (res[4] > 0) ? std::sqrt(res[3] / res[4]) : std::sqrt(res[3]);
    st->solve_ms = ms;
  }
  return ires[1];
}

}  // namespace fvc
