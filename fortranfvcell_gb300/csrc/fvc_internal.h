// fvc_internal.h -- host-side declarations shared by the translation units
// of libfvcgpu (not part of the public C ABI).
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/fvcgpu.h"

namespace fvc {

// Where the reference's SpMV adds the diagonal term (src/Matvec.f).
enum DiagMode : int { DIAG_FIRST = 0, DIAG_LAST = 1, DIAG_NONE = 2 };

// Device copy of one matrix in SELL-32 (see fvc_device.cuh).
struct DeviceMatrix {
  int n = 0;
  int nslices = 0;
  int64_t slots = 0;      // stored slots incl. padding
  int64_t nnz_off = 0;    // true off-diagonal nonzeros
  int diag_mode = 0;
  int64_t *sptr = nullptr;
  int *col = nullptr;
  double *val = nullptr;
  double *diag = nullptr;  // ad (null for DIAG_NONE)
  double *jac = nullptr;   // Jacobi m (the reference's m = ad)
  double *jinv = nullptr;  // 1/m (FP64), computed once per value upload
  // FP32 operator for mixed precision in difference form:
  //   (A x)_i = e_i x_i + sum_k w_ik (x_i - x_k),  w = -a_ik, e_i = a_ii - sum w
  float *val32 = nullptr;   // w per slot (0 on padding and on a diagonal slot)
  float *diag32 = nullptr;  // e per row (clamped to +-1e30)
  float *minv32 = nullptr;  // Jacobi 1/m per row (0 for |m| beyond FP32)
  int16_t *col16 = nullptr; // column - row per slot (when every one fits)
  uint8_t *sflag = nullptr; // per slice: 1 if some row has e_i != 0
  // set by the FP32 build when a slot that held 0 when the layout was
  // chosen (and so was given offset 0) holds a value whose offset needs
  // more than 16 bits; the mixed kernels then refuse to run
  int *f32_bad = nullptr;
  bool col16_ok = false;
  int ell_w = 0;             // FP32 copy padded to this uniform slice width (0: SELL)
  bool have32 = false;
  bool layout32 = false;     // the FP32 layout (col16_ok, ell_w, buffers) is decided
  int layout_mode = 0;       // ... for this fvc_opts.fp32_layout
  int cl_smax = -1;          // cluster PCG: most slots of one CTA's rows (-1: unknown)
  int *mirror = nullptr;     // per slot: the slot of the transposed entry (built on demand)
  // a mixed BiCGSTAB on this structure stalled: its later mixed BiCGSTAB
  // solves (new values, same structure) run in FP64 from the start
  mutable bool bcg32_stalled = false;
  // host-side description of the source layout, for value updates
  int matriz = 0, unsym = 0, nad = 0;
  int64_t *src_of_slot = nullptr;  // device map: slot -> source value index
  int8_t *src_arr = nullptr;       // device map: slot -> 0 none,1 ad,2 au,3 al
};

struct Scratch {
  size_t n = 0, nf = 0, ngmres = 0;  // capacities of v[], f[], g
  static constexpr int kVec = 10;
  double *v[kVec] = {nullptr};  // Krylov vectors
  float *f[10] = {nullptr};     // FP32 vectors (mixed precision)
  double *g = nullptr;          // GMRES basis (k+1) x n
  double *partials = nullptr;   // reduction partials
  size_t npart = 0;
  unsigned int *sync = nullptr; // barrier counter + generation
  int *err = nullptr;
  double *result = nullptr;     // solver scalars written by block 0
  int *iresult = nullptr;
  double *trace = nullptr;      // per residual replacement: (iteration, ||r||/||b||)
  float *history = nullptr;     // per iteration: recursive ||r||/||b|| (first kHistoryMax)
};

constexpr int kTraceMax = 256;
// Mixed precision: the FP32 iterations reduce the residual by this factor
// between two FP64 recomputations (CG: a reliable update; BiCGSTAB: a
// defect-correction sweep).  For BiCGSTAB, 0.1 rather than a deep inner
// solve: a restarted FP32 BiCGSTAB stalls near FP32's limit on the
// enthalpy systems (the enthalpy systems of 256 heated cavities, batched:
// 198 ms at 0.1, 291 ms at 1e-2, 693 ms at 1e-4; FP64 251 ms).
constexpr double kInnerTolDefault = 0.1;
constexpr int kHistoryMax = 16384;

struct Launch {
  int threads = 256;
  int blocks = 0;
};

// Kernel launch counter (fvc_kernel_launches).
void count_launch(int64_t k = 1);

// Krylov drivers (fvc_krylov.cu).  All synchronous on `stream`.
int32_t run_pcg(const DeviceMatrix &A, Scratch &S, const double *b, double *x,
                double tol, int maxit, int init, const fvc_opts &o,
                cudaStream_t stream, fvc_stats *st);
int32_t run_bicgstab(const DeviceMatrix &A, Scratch &S, const double *b,
                     double *x, double tol, int maxit, int init,
                     const fvc_opts &o, cudaStream_t stream, fvc_stats *st);
// BiCGSTAB on A^T x = b over A's storage (A.mirror built): FVC_ERR_UNSUPPORTED without it
int32_t run_bicgstab_transposed(const DeviceMatrix &A, Scratch &S, const double *b, double *x,
                                double tol, int maxit, int init, const fvc_opts &o,
                                cudaStream_t stream, fvc_stats *st);
int32_t run_gmres(const DeviceMatrix &A, Scratch &S, const double *b, double *x,
                  double tol, int maxit, const fvc_opts &o, cudaStream_t stream,
                  fvc_stats *st);
// PCG on one thread-block cluster (fvc_cluster.cu); FVC_ERR_UNSUPPORTED
// when the system does not fit one cluster's shared memory
int32_t run_pcg_cluster(const DeviceMatrix &A, Scratch &S, const double *b, double *x,
                        double tol, int maxit, int init, const fvc_opts &o,
                        cudaStream_t stream, fvc_stats *st);
int32_t enqueue_pcg_cluster(const DeviceMatrix &A, Scratch &S, const double *b, double *x,
                            double tol, int maxit, int init, const fvc_opts &o,
                            cudaStream_t stream, bool launch);
int cluster_slots_max(int n, int nslices, const int64_t *sptr);
// An FP64 solve (code 1..3, the kernel run_pcg / run_bicgstab / run_gmres
// would choose) enqueued on `stream` without waiting; its scalars stay on
// the device (launch_solve_status copies them out).  launch = false only
// allocates the scratch, so that a later call can be captured into a graph.
int32_t enqueue_solve(const DeviceMatrix &A, Scratch &S, int code, const double *b, double *x,
                      double tol, int maxit, int init, const fvc_opts &o, cudaStream_t stream,
                      bool launch);
// out[0..3] = status, iterations, inner iterations, timeout flag of the
// solve enqueued last on S (mixed: the iterations are the FP32 ones)
int32_t launch_solve_status(const Scratch &S, int32_t *out, cudaStream_t stream,
                            bool mixed = false);
// Batched PCG / BiCGSTAB of the block-diagonal matrix A (fvc_krylov.cu):
// codes (1 PCG, 2 BiCGSTAB), tols and its_hint (expected iterations, for
// the share of blocks) per system may be null (all PCG, all tol, sqrt of
// the rows); inits gives each system's warm-start rule.
int32_t run_krylov_batched(DeviceMatrix &A, Scratch &S, int nsys,
                           const int32_t *row_start, const int32_t *codes, const double *tols,
                           const double *its_hint, const int32_t *inits, const double *b,
                           double *x, double tol, int maxit, const fvc_opts &o,
                           cudaStream_t stream, fvc_stats *st);
// A batched launch planned once for a fixed block-diagonal structure
// (plan_batched): the systems' descriptors, their block shares and the
// launch's counters and result slots in one device buffer.  Each
// enqueue_batched zeroes the counters and results and launches, with no
// host transfer, so the launch can be captured in a CUDA graph.  run (may
// be null) is a device array of one int32 per system: 0 skips that
// system in the launch (x keeps its rows' values).
struct BatchSys;
struct BatchPlan {
  int nsys = 0, total = 0, threads = 0;
  bool mixed = false, persistent = false;
  const void *kern = nullptr;
  char *buf = nullptr;
  size_t ctr_bytes = 0, res_bytes = 0, ires_bytes = 0;
  int *err = nullptr;
  double *res = nullptr;  // 16 per system: [1] conv [2] crit [3] |b-Ax|^2 [4] |b|^2
  int *ires = nullptr;    // 16 per system: [0] iterations (mixed: updates) [1] status
                          // [2] inner iterations
  BatchSys *dsys = nullptr;
  int *dsob = nullptr;
  double tol = 0.0;
  int fp32_layout = 0;
  int cluster = 0;  // > 0: one cluster per system (cluster launches)
  // cluster launches: one per cluster size, systems of the same size
  // together; segment k covers blocks [sob_off, sob_off + blocks) of the
  // block-to-system map.  Segments after the first run on their own
  // streams, forked from and joined back to the caller's.
  static constexpr int kMaxSeg = 16;
  int nseg = 0;
  int seg_csize[kMaxSeg] = {}, seg_blocks[kMaxSeg] = {}, seg_off[kMaxSeg] = {};
  cudaStream_t aux[kMaxSeg] = {};
  cudaEvent_t fork = nullptr, join[kMaxSeg] = {};
};
int32_t plan_batched(DeviceMatrix &A, Scratch &S, int nsys, const int32_t *row_start,
                     const int32_t *codes, const double *tols, const double *its_hint,
                     const int32_t *inits, const int32_t *run, double tol, const fvc_opts &o,
                     cudaStream_t stream, bool persistent, BatchPlan &P);
int32_t enqueue_batched(DeviceMatrix &A, Scratch &S, const BatchPlan &P, const double *b,
                        double *x, int maxit, const fvc_opts &o, cudaStream_t stream);
void free_batched(BatchPlan &P, cudaStream_t stream);
// A mixed solve enqueued without waiting (launch = false: allocations,
// the FP32 layout and operator only, for a later captured call)
int32_t enqueue_mixed(const DeviceMatrix &A, Scratch &S, int code, const double *b, double *x,
                      double tol, int maxit, int init, const fvc_opts &o, cudaStream_t stream,
                      bool launch);
int32_t run_mixed(const DeviceMatrix &A, Scratch &S, int code, const double *b,
                  double *x, double tol, int maxit, int init, const fvc_opts &o,
                  cudaStream_t stream, fvc_stats *st);
int32_t launch_spmv(const DeviceMatrix &A, const double *x, double *y,
                    cudaStream_t stream, bool fused = false);
int32_t launch_reciprocal(const DeviceMatrix &A, cudaStream_t stream);
int32_t launch_spmv_f32(const DeviceMatrix &A, const float *x, float *y,
                        cudaStream_t stream);
// mode: fvc_opts.fp32_layout (0 uniform width where possible, 1 own widths)
int32_t build_f32_copy(DeviceMatrix &A, cudaStream_t stream, int mode);
int32_t ensure_f32_vectors(Scratch &S, size_t n);
// batched mixed-precision solves (fvc_mixed.cu): the kernel for the block
// size (for occupancy queries) and its cooperative launch over the batch
// descriptors (device BatchSys array) and the block-to-system map
struct BatchSys;
const void *mixed_batched_kernel(int threads);
const void *krylov_batched_kernel(int threads);
// A batched launch: groups of blocks of one cooperative launch (csize 0),
// or an ordinary launch of clusters of csize blocks
cudaError_t launch_groups(const void *kern, int blocks, int threads, int csize, void **args,
                          cudaStream_t stream);
void cluster_config(cudaLaunchConfig_t &cfg, cudaLaunchAttribute *at, int csize, int threads,
                    cudaStream_t stream);
int32_t launch_mixed_batched(const DeviceMatrix &A, const Scratch &S, const BatchSys *dsys,
                             const int *dsob, int blocks, int threads, int cluster,
                             const double *b, double *x, int maxit, const fvc_opts &o,
                             cudaStream_t stream);

// Threads per block of a persistent solver launch when the caller sets
// none (or a multiple of 128 it asked for, clamped to 128..1024).  The
// automatic choice is one block per SM with the fewest warps that still
// cover every slice: a system too small to fill the GPU with 1024-thread
// blocks spreads its rows over more SMs, because at a few thousand rows per
// SM the FP64 pipe (about two lanes per clock per SM on this GPU) and not
// the memory system sets the iteration time.  Systems of 152 x 1024 rows
// and more get 1024 threads.
inline int block_threads_for(int requested, int nslices, int sms) {
  if (requested > 0) return std::min(1024, std::max(128, requested & ~127));
  const int warps = (nslices + std::max(sms, 1) - 1) / std::max(sms, 1);
  return std::min(1024, std::max(128, (warps * 32 + 127) / 128 * 128));
}

namespace cells {
// fvc_cells_gradient without the wait: an unsupported boundary code sets
// *d_err (device) instead of being returned
int32_t gradient_async(const fvc_cell_mesh *m, int kind, int comp, const double *u,
                       double *grad, int *d_err, cudaStream_t s);
}  // namespace cells

// Allocates what fvc_solve_async needs for (code, opts) on this context.
int32_t context_prepare(fvc_context *c, int code, const fvc_opts &o);
// A persistent batched plan over the context's block-diagonal matrix, its
// capturable launch on the context's stream, and its release (BatchPlan).
int32_t context_plan_batched(fvc_context *c, int nsys, const int32_t *row_start,
                             const int32_t *codes, const double *tols, const double *its_hint,
                             const int32_t *inits, const int32_t *run, double tol,
                             const fvc_opts &o, BatchPlan &P);
int32_t context_enqueue_batched(fvc_context *c, const BatchPlan &P, const double *b, double *x,
                                int maxit, const fvc_opts &o);
void context_free_batched(fvc_context *c, BatchPlan &P);
// src/Solver.f's warm-start rule for (code, matriz): 1 zeroes x first
int context_default_init(int code, int matriz);

}  // namespace fvc
