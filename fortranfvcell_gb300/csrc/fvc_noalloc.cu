// fvc_noalloc.cu -- an allocation-free FP64 PCG for callers that cannot
// call cudaMalloc.
//
// Some callers of this solver cannot allocate device memory at solve time:
// a host code that hands the GPU a fixed memory budget up front (every byte
// accounted for at start-up, as a Fortran code with one static work vector
// like the reference's `ia(maxmem)` does), a process whose allocations are
// made once by a pool it does not control, or a call site where a
// cudaMalloc would synchronise the device in the middle of a time step.
// This entry point takes the matrix and vectors the caller already holds on
// the device and runs the solve with scratch from one file-scope device
// array instead of allocating.
//
// The kernel is the persistent Jacobi-PCG of fvc_krylov.cu
// (src/Iterativos.f:29-106 restated with FMA), reading the reference's CSRD
// arrays directly (1-based ia/ja, diagonal in ad, off-diagonals in au)
// instead of the SELL-32 copy the context API builds.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "fvc_device.cuh"
#include "fvc_internal.h"

namespace fvc {

namespace {

// Capacity of the static scratch: rows and co-resident blocks.
constexpr int kNoAllocMaxRows = 131072;
constexpr int kNoAllocMaxBlocks = 256;
constexpr int kNoAllocThreads = 1024;

// Layout of the scratch array (doubles):
//   [0, 5*R)                 r, z, p (two buffers), q
//   [5R, 5R + 4*kMaxNV*B)    reduction partials
//   then 4*kMaxNV totals, 16 results, then 16 words of counters
constexpr size_t kVecDoubles = 5 * (size_t)kNoAllocMaxRows;
constexpr size_t kPartDoubles = 4 * (size_t)kMaxNV * kNoAllocMaxBlocks;
constexpr size_t kTotDoubles = 4 * (size_t)kMaxNV;
constexpr size_t kResDoubles = 16;
constexpr size_t kCtrDoubles = 16;  // count, flag, err, iresult (as 32-bit words)
constexpr size_t kScratchDoubles = kVecDoubles + kPartDoubles + kTotDoubles + kResDoubles + kCtrDoubles;

// A device holds this array (~5.0 MiB) from the first call on it (the load
// of this module on that device) until the process exits.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct NoAllocArgs {
  const double *ad, *au;
  const int *ia, *ja;  // 1-based, as src/Datastruct.f builds them
  int n;
  const double *b;
  double *x;
  double *r, *z, *pa, *pb, *q;
  GridSync gs;
  double tol;
  int maxit, init, stop_rule;
  double *result;
  int *iresult;
};

__device__ __forceinline__ double csrd_row(const NoAllocArgs &a, int i, const double *v) {
  double t = a.ad[i] * v[i];
  const int k1 = a.ia[i + 1] - 1;
  for (int k = a.ia[i] - 1; k < k1; ++k) t = fma(a.au[k], v[a.ja[k] - 1], t);
  return t;
}

template <typename PF>
__device__ __forceinline__ double csrd_row_f(const NoAllocArgs &a, int i, PF pf) {
  double t = a.ad[i] * pf(i);
  const int k1 = a.ia[i + 1] - 1;
  for (int k = a.ia[i] - 1; k < k1; ++k) t = fma(a.au[k], pf(a.ja[k] - 1), t);
  return t;
}

// Rows are split into equal contiguous ranges per block, one row per thread
// per step.
#define NA_FOR_ROWS(n)                                                      \
  for (int row = (int)(blockIdx.x * (((n) + gridDim.x - 1) / gridDim.x)) + \
                 (int)threadIdx.x,                                          \
           end_ = min((n), (int)((blockIdx.x + 1) * (((n) + gridDim.x - 1) / gridDim.x))); \
       row < end_; row += blockDim.x)

// Status the kernel reports when the structure check fails.
constexpr int kBadStructure = -1;

__global__ void __launch_bounds__(kNoAllocThreads, 1) pcg_csrd_noalloc_kernel(NoAllocArgs a) {
  __shared__ double red[kMaxNV * 32];
  const int n = a.n;
  unsigned int ep = 0;
  // Structure check before any gather: ia(1) = 1, each row's length in
  // [0, n-1], every column in [1, n]; and at least one entry above the
  // diagonal when there are off-diagonals at all.  Symmetric CSRD keeps
  // only the strictly lower triangle (src/Datastruct.f:77, matvec_csrd_sym
  // src/Matvec.f:216-250); applied as unsymmetric CSRD it would be a
  // different operator, so such input is refused rather than solved wrongly.
  double chk[3] = {0.0, 0.0, 0.0};  // bad rows, entries above, off-diagonals
  NA_FOR_ROWS(n) {
    const int k0 = a.ia[row], k1 = a.ia[row + 1];
    const bool ok_row = (row > 0 || k0 == 1) && k0 >= 1 && k1 >= k0 && k1 - k0 <= n - 1;
    if (!ok_row) {
      chk[0] += 1.0;
      continue;
    }
    for (int k = k0 - 1; k < k1 - 1; ++k) {
      const int c = a.ja[k];
      if (c < 1 || c > n) {
        chk[0] += 1.0;
        break;
      }
      if (c - 1 > row) chk[1] += 1.0;
    }
    chk[2] += (double)(k1 - k0);
  }
  if (!grid_allreduce<3>(a.gs, ep, chk, red)) return;
  if (chk[0] != 0.0 || (chk[2] > 0.0 && chk[1] == 0.0)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.iresult[0] = 0;
      a.iresult[1] = kBadStructure;
      a.result[1] = chk[0];
    }
    return;
  }
  double acc[2] = {0.0, 0.0};
  NA_FOR_ROWS(n) {
    double ax;
    if (a.init) {
      ax = 0.0;
      a.x[row] = 0.0;
    } else {
      ax = csrd_row(a, row, a.x);
    }
    const double ri = a.b[row] - ax;
    const double zi = ri / a.ad[row];
    a.r[row] = ri;
    a.pa[row] = zi;
    acc[0] = fma(ri, zi, acc[0]);
    acc[1] = fma(a.b[row], a.b[row], acc[1]);
  }
  if (!grid_allreduce<2>(a.gs, ep, acc, red)) return;
  double d = acc[0];
  const double conv = (a.stop_rule == 0) ? a.tol * sqrt(fabs(d)) : a.tol * sqrt(acc[1]);
  double beta = 0.0, crit = 0.0;
  double *pprev = a.pa, *pcur = a.pa;
  int j, status = FVC_OK;
  for (j = 1; j <= a.maxit; ++j) {
    double pq[1] = {0.0};
    if (j == 1) {
      NA_FOR_ROWS(n) {
        const double qi = csrd_row(a, row, pcur);
        a.q[row] = qi;
        pq[0] = fma(pcur[row], qi, pq[0]);
      }
    } else {
      const double *pp = pprev;
      const double *z = a.z;
      NA_FOR_ROWS(n) {
        auto pf = [&](int k) { return fma(beta, pp[k], z[k]); };
        const double pi = pf(row);
        pcur[row] = pi;
        const double qi = csrd_row_f(a, row, pf);
        a.q[row] = qi;
        pq[0] = fma(pi, qi, pq[0]);
      }
    }
    if (!grid_allreduce<1>(a.gs, ep, pq, red)) return;
    const double alpha = d / pq[0];
    acc[0] = 0.0;
    acc[1] = 0.0;
    NA_FOR_ROWS(n) {
      a.x[row] = fma(alpha, pcur[row], a.x[row]);
      const double ri = fma(-alpha, a.q[row], a.r[row]);
      const double zi = ri / a.ad[row];
      a.r[row] = ri;
      a.z[row] = zi;
      acc[0] = fma(ri, zi, acc[0]);
      acc[1] = fma(ri, ri, acc[1]);
    }
    if (!grid_allreduce<2>(a.gs, ep, acc, red)) return;
    beta = acc[0] / d;
    d = beta * d;
    crit = (a.stop_rule == 0) ? sqrt(fabs(d)) : sqrt(acc[1]);
    if (!(crit == crit) || isinf(d)) {
      status = FVC_ERR_NAN;
      break;
    }
    if (crit < conv) break;
    pprev = pcur;
    pcur = (pcur == a.pa) ? a.pb : a.pa;
  }
  if (j > a.maxit) {
    j = a.maxit;
    status = FVC_ERR_NOCONV;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.iresult[0] = j;
    a.iresult[1] = status;
    a.result[1] = conv;
    a.result[2] = crit;
  }
}

// Device address of g_noalloc_scratch on the current device.  Host code
// cannot use the array's name as an address, so it asks the runtime, on
// every call: the address belongs to the module loaded in the device's
// current context, and a context that was reset and re-created (a
// cudaDeviceReset in between) loads the module again, possibly elsewhere.
// Once the module is loaded the look-up allocates nothing.  Under CUDA's
// lazy module loading (CUDA_MODULE_LOADING=LAZY, the default since
// CUDA 12.2) the first look-up on a device is what loads the module, and
// with it places the array in device memory.
int32_t noalloc_scratch(double **out) {
  void *p = nullptr;
  const cudaError_t ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (ce != cudaSuccess || !p) {
    fprintf(stderr, "fvc_pcg_csrd_noalloc: cudaGetSymbolAddress failed: %s\n",
            cudaGetErrorString(ce));
    return FVC_ERR_CUDA;
  }
  *out = static_cast<double *>(p);
  return FVC_OK;
}

}  // namespace

}  // namespace fvc

extern "C" int32_t fvc_pcg_csrd_noalloc(const double *d_ad, const double *d_au,
                                        const int32_t *d_ia, const int32_t *d_ja, int32_t neq,
                                        const double *d_b, double *d_x, double tol,
                                        int32_t maxit, int32_t init, int32_t stop_rule,
                                        void *stream, fvc_stats *stats) {
  using namespace fvc;
  if (stats) memset(stats, 0, sizeof(*stats));
  if (!d_ad || !d_au || !d_ia || !d_ja || !d_b || !d_x || neq <= 0 || maxit < 1 ||
      (stop_rule != 0 && stop_rule != 1))
    return FVC_ERR_ARG;
  if (neq > kNoAllocMaxRows) {
    fprintf(stderr,
            "fvc_pcg_csrd_noalloc: neq = %d exceeds the static scratch capacity of %d rows; "
            "use fvc_solve for larger systems\n",
            neq, kNoAllocMaxRows);
    return FVC_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FVC_ERR_CUDA;
  double *base = nullptr;
  int32_t rc = noalloc_scratch(&base);
  if (rc != FVC_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  int sms = 1, occ = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pcg_csrd_noalloc_kernel,
                                                    kNoAllocThreads, 0) != cudaSuccess ||
      occ <= 0)
    return FVC_ERR_CUDA;
  const int want = (neq + kNoAllocThreads - 1) / kNoAllocThreads;
  const int blocks = std::max(1, std::min(std::min(occ * sms, kNoAllocMaxBlocks), want));

  NoAllocArgs a{};
  a.ad = d_ad;
  a.au = d_au;
  a.ia = d_ia;
  a.ja = d_ja;
  a.n = neq;
  a.b = d_b;
  a.x = d_x;
  const size_t R = kNoAllocMaxRows;
  a.r = base;
  a.z = base + R;
  a.pa = base + 2 * R;
  a.pb = base + 3 * R;
  a.q = base + 4 * R;
  double *part = base + kVecDoubles;
  double *tot = part + kPartDoubles;
  double *res = tot + kTotDoubles;
  unsigned int *ctr = reinterpret_cast<unsigned int *>(res + kResDoubles);
  a.gs.partials = part;
  a.gs.totals = tot;
  a.gs.count = ctr;
  a.gs.flag = ctr + 8;
  a.gs.err = reinterpret_cast<int *>(ctr + 16);
  a.gs.nblocks = (unsigned int)blocks;
  a.iresult = reinterpret_cast<int *>(ctr + 20);
  a.result = res;
  a.tol = tol;
  a.maxit = maxit;
  a.init = init ? 1 : 0;
  a.stop_rule = stop_rule;
  // The array keeps the previous call's contents: counters, flags, error
  // word and results must start at zero (vectors are written before use).
  if (cudaMemsetAsync(ctr, 0, kCtrDoubles * sizeof(double), s) != cudaSuccess ||
      cudaMemsetAsync(res, 0, kResDoubles * sizeof(double), s) != cudaSuccess)
    return FVC_ERR_CUDA;
  void *args[] = {&a};
  if (cudaLaunchCooperativeKernel((const void *)pcg_csrd_noalloc_kernel, dim3(blocks),
                                  dim3(kNoAllocThreads), args, 0, s) != cudaSuccess)
    return FVC_ERR_CUDA;
  count_launch();
  double hres[kResDoubles];
  int hctr[24];
  if (cudaMemcpyAsync(hres, res, sizeof(hres), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(hctr, ctr, sizeof(hctr), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return FVC_ERR_CUDA;
  if (hctr[16] != 0) return FVC_ERR_TIMEOUT;
  if (hctr[21] == kBadStructure) {
    fprintf(stderr,
            "fvc_pcg_csrd_noalloc: the CSRD structure is not unsymmetric CSRD "
            "(%.0f rows with ia out of order or a column outside [1, %d], or no entry above "
            "the diagonal: symmetric lower-only storage); nothing was solved\n",
            hres[1], neq);
    return FVC_ERR_ARG;
  }
  if (stats) {
    stats->status = hctr[21];
    stats->iterations = hctr[20];
    stats->conv = hres[1];
    stats->final_crit = hres[2];
  }
  return hctr[21];
}
