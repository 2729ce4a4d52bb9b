/*
 * fvcgpu.h -- C ABI of the GB300 linear-solver library (libfvcgpu.so).
 *
 * This is the drop-in boundary for the linear-solver hot path of the
 * fortranFVCell finite-volume code: the `solver` subroutine of
 * src/Solver.f:28-29 and the routines it calls (src/Iterativos.f,
 * src/Matvec.f).  Plain pointers and sizes only; no C++ or torch types.
 *
 * Conventions shared by every entry point (as in the reference):
 *   - indices (iax, ja, num, nelcon, id) are Fortran 1-based values;
 *   - off-diagonal matrix values are stored NEGATED (A = diag - neighbours),
 *     exactly as the reference's assembly writes them (src/Csr.f:172,
 *     src/EllPack.f:85);
 *   - matriz: 1 CSRD, 2 CSR, 3 CSRC, 4 ELLPACK (src/Datastruct.f:27-179);
 *   - code:   1 PCG, 2 BiCGSTAB, 3 GMRES(15)   (src/Solver.f:19-21).
 */
#ifndef FVCGPU_H
#define FVCGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  FVC_OK = 0,
  FVC_ERR_NOCONV = 1,      /* maxit reached (reference: print + STOP)      */
  FVC_ERR_BREAKDOWN = 2,   /* a Krylov denominator became exactly zero     */
  FVC_ERR_NAN = 3,         /* NaN/Inf in the iteration                     */
  FVC_ERR_UNSUPPORTED = 4, /* code x matriz pair the reference rejects     */
  FVC_ERR_CUDA = 5,        /* CUDA runtime error or no usable GPU          */
  FVC_ERR_ARG = 6,         /* invalid argument                             */
  FVC_ERR_TIMEOUT = 7      /* an on-device wait exceeded its bound         */
};

/* ---- drop-in solver ---------------------------------------------------- */
/* Replaces src/Solver.f:28-346 `solver(ad,au,al,x,b,iax,ja,neq,nad,unsym,
 * tol,maxit,code,matriz,nlit)`.  Every argument is passed by reference as
 * gfortran passes it; `unsym` is a Fortran LOGICAL (4 bytes, nonzero =
 * .true.).  All arrays are host arrays owned by the caller.
 *
 * Behaviour follows the reference path that Solver.f selects for the same
 * (code, matriz, unsym) when openmpSolver is .false.: the warm-start rule
 * (x zeroed or used as the initial guess), the Jacobi preconditioner
 * m = ad, and the stopping tests of src/Iterativos.f.  Differences:
 *   - b is left unchanged (the reference overwrites it with p or s);
 *   - non-convergence prints the reference's warning and, like Fortran
 *     STOP, ends the process unless FVC_STOP_ON_ERROR=0 is set in the
 *     environment, in which case the call returns with x = last iterate.
 * Unsupported pairs (BiCGSTAB/GMRES with matriz 2, src/Solver.f:224-227,
 * 305-308; unknown code, :337-339) print the reference's message and stop
 * the same way. */
void fvc_solver(double *ad, double *au, double *al, double *x, double *b,
                const int32_t *iax, const int32_t *ja, const int32_t *neq,
                const int32_t *nad, const int32_t *unsym, const double *tol,
                const int32_t *maxit, const int32_t *code,
                const int32_t *matriz, const int32_t *nlit);

/* Same as fvc_solver, under the gfortran-mangled name of the reference
 * subroutine, so object files compiled from the reference link against this
 * library unchanged once src/Solver.f is left out of the build. */
void solver_(double *ad, double *au, double *al, double *x, double *b,
             const int32_t *iax, const int32_t *ja, const int32_t *neq,
             const int32_t *nad, const int32_t *unsym, const double *tol,
             const int32_t *maxit, const int32_t *code, const int32_t *matriz,
             const int32_t *nlit);

/* ---- extended solver --------------------------------------------------- */
enum {
  FVC_PREC_FP64 = 0,  /* reference arithmetic: FP64 everywhere             */
  FVC_PREC_MIXED = 1  /* FP32 SpMV + Jacobi inside FP64 defect correction  */
  /* A mixed BiCGSTAB whose sweeps stop cutting the FP64 residual (three in a
   * row each below a tenth) ends its FP32 part early; fvc_solve and the
   * drop-in then finish in FP64 BiCGSTAB from that iterate (stats: the
   * iterations of both parts, the FP32 ones in inner_iterations), and the
   * context's later mixed BiCGSTAB solves run in FP64 from the start until
   * fvc_matrix_set gives it another structure.  fvc_solve_async reports
   * that stall as FVC_ERR_NOCONV and, after one in an fvc_solve of the
   * context, routes later ones to FP64 too; fvc_solve_batched finishes the
   * stalled systems in FP64 in a second launch; the SIMPLE batch
   * (fvc_simple_batch_*) finishes them in FP64 inside its graph. */
};

typedef struct {
  int32_t precision;   /* FVC_PREC_*                                       */
  int32_t init;        /* -1: the reference's rule for (code,matriz); 0: warm
                          start from x; 1: start from x = 0               */
  double refine_tol;   /* MIXED: target ||b-Ax||/||b|| (0 -> derived: tol)  */
  double inner_tol;    /* MIXED: FP32 reduction of the residual between two
                          FP64 residual recomputations (0 -> 0.1)      */
  int32_t max_refine;  /* MIXED: max outer sweeps (0 -> 30)                */
  int32_t block_threads; /* 0 -> autotuned                                 */
  int32_t blocks_per_sm; /* 0 -> autotuned                                 */
  int32_t stop_rule;   /* 0: the reference's test for the method;
                          1: ||r||2 <= tol*||b||2 on the recurrence residual */
  int32_t want_residual; /* 1: recompute ||b-Ax||/||b|| in FP64 at exit   */
  int32_t update_beta; /* MIXED CG: beta = (r.z)/(r_old.z_old) at a residual
                          replacement taken from 0: the replaced (true)
                          residual; 1: the recursive one                 */
  int32_t staging;     /* MIXED CG: 0 streams the iteration's arrays through
                          shared memory with bulk asynchronous copies when
                          the layout allows (1024 threads, 16-bit column
                          offsets) and the system has 524288 rows or more;
                          1: plain loads; 2: staged whenever the layout
                          allows                                           */
  int32_t max_blocks;  /* cap on the persistent grid (0 -> automatic)      */
  int32_t fp32_layout; /* MIXED: the FP32 operator's slice widths.  0: when
                          no row has more than 4 off-diagonals, every slice
                          padded to the widest (width 3 or 4: no slice
                          pointers, the staged kernels' uniform form), else
                          each slice its own width; 1: each slice its own
                          width (SELL-32: no padding slots, slice pointers).
                          A solve that asks for the other choice than the
                          context's operator has lays it out anew (a host
                          wait), so graphs captured before then are stale */
  int32_t cluster_size; /* batched solves: how each system's blocks work
                          together.  1: a group of blocks of one cooperative
                          launch, synchronised through global memory, the
                          share of blocks by expected work; k in 2..16: one
                          thread-block cluster of k blocks per system
                          (cluster barrier and distributed shared memory;
                          an ordinary launch whose clusters start as SMs
                          free up, heaviest systems first; above 8 needs
                          the non-portable cluster sizes); -1: one cluster
                          per system sized to it (ceil(rows / r) blocks, r
                          the largest system's rows / 16, at least 1024;
                          one launch per size, the launches side by side on
                          forked streams); 0: automatic -- -1 when the
                          systems' clusters would fill the device (their
                          blocks at least its resident 256-thread
                          blocks), else 1.  Single solves ignore it     */
} fvc_opts;

typedef struct {
  int32_t status;      /* FVC_*                                            */
  int32_t iterations;  /* j of the reference loop at exit (GMRES: cycles)  */
  int32_t inner_iterations; /* GMRES inner steps; MIXED: total FP32 its   */
  int32_t refinements; /* MIXED: outer sweeps                              */
  double energy;       /* x.Ax (PCG/BiCGSTAB) or x.b (GMRES), as logged in
                          the reference's unit-13 line                     */
  double conv;         /* the stopping threshold                           */
  double final_crit;   /* the stopped quantity at exit                     */
  double rel_residual; /* ||b-Ax||/||b|| recomputed in FP64 (if requested) */
  double solve_ms;     /* device time of the solve                         */
} fvc_stats;

void fvc_opts_default(fvc_opts *opts);

/* Host-array solve with explicit options; returns an FVC_* status and never
 * ends the process.  Arguments by value; arrays as in fvc_solver. */
int32_t fvc_solver_ex(double *ad, double *au, double *al, double *x,
                      const double *b, const int32_t *iax, const int32_t *ja,
                      int32_t neq, int32_t nad, int32_t unsym, double tol,
                      int32_t maxit, int32_t code, int32_t matriz,
                      const fvc_opts *opts, fvc_stats *stats);

/* ---- device-resident context ------------------------------------------ */
/* A context owns the device copy of one matrix and its solver scratch, so a
 * caller that solves the same structure repeatedly (one SIMPLE outer
 * iteration after another) uploads the structure once.  Not thread-safe;
 * use one context per host thread. */
typedef struct fvc_context fvc_context;

int32_t fvc_context_create(fvc_context **ctx, int32_t device);
int32_t fvc_context_destroy(fvc_context *ctx);
/* cudaStream_t passed as void*; NULL = the legacy default stream */
int32_t fvc_context_set_stream(fvc_context *ctx, void *stream);

/* Load a matrix in reference layout from HOST arrays (conversion to the
 * device layout happens here).  au/al may be NULL where matriz/unsym do not
 * use them (see src/Datastruct.f). */
int32_t fvc_matrix_set(fvc_context *ctx, int32_t matriz, int32_t unsym,
                       int32_t neq, int32_t nad, const double *ad,
                       const double *au, const double *al, const int32_t *iax,
                       const int32_t *ja);
/* Replace only the values (same structure as the last fvc_matrix_set). */
int32_t fvc_matrix_update_values(fvc_context *ctx, const double *ad,
                                 const double *au, const double *al);

/* Solve with DEVICE vectors b (not modified) and x (in: guess, out: solution)
 * on the context's stream.  Synchronous: returns after the solve ends. */
int32_t fvc_solve(fvc_context *ctx, int32_t code, const double *d_b, double *d_x,
                  double tol, int32_t maxit, const fvc_opts *opts,
                  fvc_stats *stats);

/* Solve the transposed system A^T x = b (DEVICE vectors, as fvc_solve)
 * with the reference's Jacobi BiCGSTAB (code 2; src/Iterativos.f:140-234)
 * over the context's stored matrix: the SpMV reads entry (i, j) of A^T as
 * the stored value of (j, i) through a per-slot mirror index built at the
 * first call for a structure.  There is no transposed copy of the values,
 * so a value update of A serves both A and A^T.  The Jacobi preconditioner
 * is A's diagonal, which A^T shares.  The adjoint solves of
 * fortranfvcell_gb300.autograd use it.  FVC_ERR_UNSUPPORTED for other
 * codes, FVC_PREC_MIXED, matriz 2, or an off-diagonal pattern that is not
 * symmetric (every cell-adjacency structure of the reference is). */
int32_t fvc_solve_transposed(fvc_context *ctx, int32_t code, const double *d_b,
                             double *d_x, double tol, int32_t maxit,
                             const fvc_opts *opts, fvc_stats *stats);

/* fvc_matrix_update_values without the wait: the copies and the value
 * gather are enqueued on the context's stream.  With DEVICE value arrays the
 * call can be recorded in a CUDA stream capture on that stream. */
int32_t fvc_matrix_update_values_async(fvc_context *ctx, const double *ad,
                                       const double *au, const double *al);

/* fvc_solve without the wait, for CUDA graphs: the same kernels, and so
 * the same results, enqueued on the context's stream.  The call makes no
 * host-device copy and no synchronisation, so it can be recorded in a
 * stream capture on that stream and replayed.  When the solve has run,
 * d_status (DEVICE, 4 int32) holds the FVC_* status, the iterations, the
 * inner iterations (GMRES steps) and 1 if an on-device wait gave up
 * (status FVC_ERR_TIMEOUT); with FVC_PREC_MIXED the iterations are the FP32
 * ones.  A mixed BiCGSTAB that stalls here is not finished in FP64: d_status
 * holds FVC_ERR_NOCONV.  Once an fvc_solve on the context has met such a
 * stall (and finished it in FP64), this call, like fvc_solve, runs the
 * later mixed BiCGSTAB solves of that structure as FP64 BiCGSTAB to the
 * mixed target on ||r||2/||b||2, until fvc_matrix_set gives it a new
 * structure.  The first call for a context, precision and launch shape allocates
 * work buffers (and lays out the FP32 operator), so it must not be the
 * captured one.  Returns FVC_OK once the work is enqueued;
 * FVC_ERR_UNSUPPORTED for mixed GMRES and for the (code, matriz) pairs
 * fvc_solve rejects. */
int32_t fvc_solve_async(fvc_context *ctx, int32_t code, const double *d_b,
                        double *d_x, double tol, int32_t maxit,
                        const fvc_opts *opts, int32_t *d_status);

/* Launch-shape autotuner: times trial solves of trial_its iterations (b =
 * 1, x = 0, no early stop) of the context's matrix with code and precision
 * over the shapes the kernels support -- the automatic choice (a thread-
 * block cluster for a PCG system of at most 8192 rows, else one block per
 * SM with the fewest warps that cover the rows), 128..1024 threads per
 * block, a cap of 16/38/76 blocks, for mixed CG plain loads or the
 * staged copies at 1024 threads, and for mixed solves the FP32 operator's
 * slice widths (fvc_opts.fp32_layout: every slice padded to the widest row,
 * or each slice its own width) -- and writes the fastest per iteration to
 * *best (init -1, the rest as fvc_opts_default) and its time to *best_us
 * (may be NULL).  Pass *best to fvc_solve for later solves of this matrix
 * and method.  The shape changes only the summation order of the
 * reductions, so results move at rounding level; the slice width changes
 * nothing (padding slots add exactly 0).  Rows are one lane each in 32-row
 * slices: with 3 or 4 off-diagonals per row, two lanes per row would leave
 * half of every load on padding, so that is not tuned.  Returns FVC_OK, or
 * an FVC_* error; FVC_ERR_UNSUPPORTED for the (code, matriz) pairs
 * fvc_solve rejects and for mixed GMRES. */
int32_t fvc_autotune(fvc_context *ctx, int32_t code, int32_t precision,
                     int32_t trial_its, fvc_opts *best, double *best_us);

/* Batched Jacobi-PCG (src/Iterativos.f:29-106) of nsys independent systems
 * in one persistent launch: the context's matrix holds them block-
 * diagonally, system s on rows row_start[s] .. row_start[s+1]-1 (host
 * array of nsys+1 entries, row_start[0] = 0, row_start[nsys] = neq, every
 * start a multiple of 32).  Rows that pad a system to the next start must
 * be identity rows with b = 0 and x = 0.  Each system runs on its own group
 * of blocks with its own reductions and stopping test (tol, maxit and the
 * warm-start rule as in fvc_solve with code 1), so the iteration counts of
 * the systems are independent.  opts->cluster_size chooses the groups: one
 * thread-block cluster per system (mixed precision by default), or blocks
 * of one cooperative launch sharing the device by expected work (FP64 by
 * default), where nsys is limited to the co-resident blocks of the launch
 * (FVC_ERR_ARG beyond).  st (host, nsys entries, may be NULL) receives
 * each system's statistics; solve_ms is the device time of the solve.
 * Returns FVC_OK when every system converged, else FVC_ERR_NAN if one broke
 * down or the first other failure.  With FVC_PREC_MIXED each system runs
 * the mixed-precision solve of fvc_solve (FP32 iterations inside FP64
 * residual replacement or defect correction, stopping on the FP64
 * ||b-Ax||/||b|| <= tol); its statistics then count the FP32 iterations
 * and the refinements.  A mixed BiCGSTAB system whose FP32 sweeps stall is
 * finished in FP64 from its iterate (on ||r||2 <= tol ||b||2), as in
 * fvc_solve, in a second launch over the stalled systems alone; its
 * iterations then add the FP64 ones to inner_iterations (the FP32 ones).
 * No counterpart in the reference, which solves one system per call
 * (src/Solver.f:28-346). */
int32_t fvc_solve_batched(fvc_context *ctx, int32_t nsys, const int32_t *row_start,
                          const double *d_b, double *d_x, double tol,
                          int32_t maxit, const fvc_opts *opts, fvc_stats *st);

/* fvc_solve_batched with a solver and a tolerance per system, so that the
 * u, v, T and p' systems of a SIMPLE outer iteration (of one case or of many)
 * go into one launch: codes[s] = 1 (Jacobi-PCG, src/Iterativos.f:29-106) or
 * 2 (Jacobi-BiCGSTAB, src/Iterativos.f:140-234); tols[s] the system's
 * stopping tolerance; its_hint[s] the iterations the system is expected to
 * take (in a SIMPLE loop, its count in the previous outer iteration), which
 * sets its share of the launch's blocks: work = slices x iterations x SpMVs
 * per iteration.  Host arrays of nsys entries; NULL codes = all PCG, NULL
 * tols = tol for all, NULL its_hint (or an entry <= 0) = sqrt(rows).  The
 * hint moves only the speed, never the results beyond rounding.  Each
 * system takes the warm-start rule of its solver (src/Solver.f) unless opts
 * sets init.  FVC_ERR_UNSUPPORTED for BiCGSTAB on matriz 2, as fvc_solve. */
int32_t fvc_solve_batched_ex(fvc_context *ctx, int32_t nsys, const int32_t *row_start,
                             const int32_t *codes, const double *tols,
                             const double *its_hint, const double *d_b, double *d_x,
                             double tol, int32_t maxit, const fvc_opts *opts,
                             fvc_stats *st);

/* y = A x with DEVICE vectors, the reference's summation order, FP64
 * (bit-identical to src/Matvec.f for the loaded format).  Asynchronous on
 * the context's stream. */
int32_t fvc_spmv(fvc_context *ctx, const double *d_x, double *d_y);
/* y = A x, FP64, the same terms in the same order with fused
 * multiply-adds (what the FP64 solvers run); within rounding of fvc_spmv.
 * Asynchronous on the context's stream. */
int32_t fvc_spmv_fast(fvc_context *ctx, const double *d_x, double *d_y);
/* y = A x with the FP32 operator of MIXED solves (difference form
 * y_i = e_i x_i + sum_k w_ik (x_i - x_k), w = -a_ik, e_i = a_ii - sum w),
 * FP32 vectors; asynchronous. */
int32_t fvc_spmv_f32(fvc_context *ctx, const float *d_x, float *d_y);

/* Convergence record of the last MIXED CG solve on this context: for each
 * residual replacement (at most max, and at most 256) the inner iteration
 * and the recomputed FP64 ||b-Ax||/||b||.  Returns the number of records,
 * or a negative FVC_* status. */
int32_t fvc_solve_trace(const fvc_context *ctx, int32_t max, int32_t *its,
                        double *relres);

/* Convergence history of the last MIXED CG solve on this context: the
 * recursive ||r||/||b|| after each iteration (the first 16384 iterations,
 * at most max).  Returns the number of values or a negative FVC_* status. */
int32_t fvc_solve_history(const fvc_context *ctx, int32_t max, float *relres);

/* Describe the device layout: rows, stored off-diagonal slots (with
 * padding), true off-diagonal nonzeros, slice count. */
int32_t fvc_matrix_info(const fvc_context *ctx, int64_t *n, int64_t *slots,
                        int64_t *nnz_off, int64_t *nslices);

/* ---- the reference's solver log --------------------------------------- */
/* After each solve (fvc_solver, solver_, fvc_solver_ex, fvc_solve) fn
 * receives the line the reference writes to its unit-13 solver log
 * (src/Iterativos.f:91-93, 216-218, 429-431; format
 * (a,a,i9,a,d20.10,a,d20.10)), e.g.
 * "PCG:       it      123 energy norm   0.1234567890D+01 tol   0.1000000000D-07".
 * The iterations and energy are those of fvc_stats.  NULL turns it off.
 * The callback runs on the calling thread, after the solve has ended. */
typedef void (*fvc_log_fn)(const char *line, void *user);
void fvc_set_solver_log(fvc_log_fn fn, void *user);

/* The same line for given values into buf (len bytes, NUL-terminated;
 * 96 suffice).  Returns its length, or -FVC_ERR_ARG. */
int32_t fvc_format_solver_log(int32_t code, int32_t iterations, double energy,
                              double tol, char *buf, int32_t len);

/* Number of kernels this library launched since load (instrumentation). */
int64_t fvc_kernel_launches(void);

/* ---- allocation-free solve --------------------------------------------- */
/* No counterpart in the reference.  FP64 Jacobi-PCG (the method of
 * fvc_solve with code 1) on a CSRD matrix (matriz 1, unsym: ad(neq), au(nad),
 * 1-based ia(neq+1)/ja(nad)) that the caller already holds in DEVICE memory,
 * with b, x also device pointers (x: initial guess unless init, then the
 * solution).  For callers that cannot allocate device memory at solve time
 * (a fixed device budget handed out at start-up, allocations owned by a
 * pool outside the caller, or a time step that must not synchronise on a
 * cudaMalloc): it calls no cudaMalloc/cudaFree.  Its scratch is one static
 * device array of about 5.0 MiB; neq above 131072 is rejected with
 * FVC_ERR_ARG and a message.  The array is placed in a device's memory when
 * this library's module is loaded on that device.  Under CUDA's lazy module
 * loading (the default) that is the first call of this function there, so
 * make one call per device during start-up, before the memory budget is
 * handed out and before any stream capture; later calls allocate nothing.
 * Every call looks the array's address up again (no cached address
 * outlives a device reset).  The structure is checked on the device before
 * any gather: ia(1) = 1, row lengths in [0, neq-1], columns in [1, neq],
 * and some entry above the diagonal; a symmetric CSRD (strictly lower part
 * only) or a broken structure returns FVC_ERR_ARG without solving.  All
 * calls share the array, so calls that overlap on the GPU (two streams, two
 * host threads) race; the call is synchronous on `stream` (a cudaStream_t,
 * NULL = default stream).  stop_rule 0 or 1 as in fvc_opts.  Returns an
 * FVC_* status; stats may be NULL. */
int32_t fvc_pcg_csrd_noalloc(const double *d_ad, const double *d_au,
                             const int32_t *d_ia, const int32_t *d_ja,
                             int32_t neq, const double *d_b, double *d_x,
                             double tol, int32_t maxit, int32_t init,
                             int32_t stop_rule, void *stream,
                             fvc_stats *stats);

/* ---- mesh -> equation graph (host) ------------------------------------- */
/* Face-neighbour table.  ix(ld,numel) column-major holds each cell's nodes
 * (1-based, counter-clockwise) in its first slots; a cell has nsides =
 * the number of nonzero leading entries (3 or 4, up to nshared).
 * nelcon(nshared,numel): neighbour cell across side i, -1 on the boundary
 * or for unused sides.  For one-type meshes this equals
 * src/Adjacency.f:1-189 (adjtria3/adjquad4).  Returns FVC_* status. */
int32_t fvc_mesh_adjacency(const int32_t *ix, int32_t ld, int32_t nnode,
                           int32_t numel, int32_t nshared, int32_t *nelcon);

/* Reverse Cuthill-McKee cell permutation: num(old cell) = new equation.
 * Same result as src/Reord.f:6-52 (SPARSPAK genrcm/fnroot/rcm with the
 * reference's tie rules); freord = 0 gives the identity. */
int32_t fvc_mesh_rcm(const int32_t *nelcon, int32_t numel, int32_t nshared,
                     int32_t freord, int32_t *num);

/* id(j, num(c)) = num(nelcon(j,c)) or -1 (src/Numeq.f:4-25). */
int32_t fvc_mesh_numeq(const int32_t *num, const int32_t *nelcon,
                       int32_t numel, int32_t nshared, int32_t *id);

/* Sparse structure for one system (src/Datastruct.f:27-179, src/Csr.f,
 * src/EllPack.f, src/Graph.f).  Call with ja == NULL to get nad (and the
 * ja length: nad for CSR formats, nshared*neq for ELLPACK), then again
 * with ja sized accordingly.  ia holds neq+1 entries (2 for ELLPACK). */
int32_t fvc_mesh_datastruc(const int32_t *id, int32_t neq, int32_t nshared,
                           int32_t matriz, int32_t unsym, int32_t *ia,
                           int32_t *ja, int32_t *nad, int64_t *ja_len);

/* ---- face-coefficient assembly (GPU) ----------------------------------- */
/* Pressure-correction (p') diffusion coefficients of
 * src/CellibPressure.f:476-572 (iws = 1) with the geometry of
 * src/Celllib.f:695-794 and src/Celllib.f:596-655, computed on the GPU one
 * thread per cell, scattered into the matrix slots of `matriz`
 * (src/Csr.f:142-227 / src/EllPack.f:68-93).
 * Inputs (host): coor(2,nnode); ix(ld,numel) as for fvc_mesh_adjacency;
 * nelcon(nshared,numel); num(numel); k(numel) the property kf per cell;
 * d(2,numel) the SIMPLE d per cell; pin_cell (1-based, 0 = none) gets the
 * 1e60 pressure pin of CellibPressure.f:557; int_vel selects the face
 * interpolation (1..3 Darwish et al., 5 Ferziger-Peric).
 * Outputs (host): ad(neq), off-diagonal values into au (CSRD/ELLPACK) in
 * the slots of (ia, ja) built by fvc_mesh_datastruc. */
int32_t fvc_assemble_pressure(const double *coor, int32_t nnode,
                              const int32_t *ix, int32_t ld, int32_t numel,
                              int32_t nshared, const int32_t *nelcon,
                              const int32_t *num, const double *kprop,
                              const double *dsimple, int32_t pin_cell,
                              int32_t int_vel, int32_t matriz, int32_t unsym,
                              const int32_t *ia, const int32_t *ja, double *ad,
                              double *au);

/* ---- SIMPLE outer-iteration cells (GPU, one thread per cell) ------------
 * The isothermal incompressible cell routines of the SIMPLE loop
 * (src/Simple.f:299-660), each reproducing the reference's arithmetic bit
 * for bit.  All pointers are DEVICE pointers; arrays keep the reference's
 * Fortran layouts; `stream` is a cudaStream_t (NULL: the default stream).
 * Cell fields are cell-ordered (1..numel), systems equation-ordered (num).
 * Boundary codes per face (pedge): 0 wall, 1 moving wall, 2 prescribed
 * velocity, 3 prescribed pressure, 4 locally parabolic; pedge(nshared+1,c)
 * = -1 pins the cell's p', -2 fixes its velocity (1e60 diagonals). */
typedef struct {
  int32_t numel, nshared, nnode, nmat;
  const double *coor;     /* (2, nnode)                                      */
  const int32_t *ix;      /* (nshared+1, numel): 1-based nodes, 0 unused;
                             row nshared+1 the material                      */
  const int32_t *nelcon;  /* (nshared, numel): face neighbours, -1 boundary  */
  const int32_t *num;     /* (numel): equation of each cell                  */
  const int32_t *pedge;   /* (nshared+1, numel): boundary codes              */
  const double *sedge;    /* (3, nshared+1, numel): boundary values u, v, p  */
  const double *e;        /* (10, nmat): e(1) viscosity, e(2) density,
                             e(6) time coefficient, e(7) TVD limiter 1..7    */
  const void *geometry;   /* optional: the mesh's cell geometry from
                             fvc_cells_geometry_create (NULL: each cell kernel
                             computes its cell's geometry from coor, as the
                             reference's cell routines do; both give the same
                             bits, the cache saves the FP64 work)            */
} fvc_cell_mesh;

/* The geometry of every cell of m (centroids, face normals, lengths and
 * midpoints, ghost centroids, the reference's cellGeom2D / vectorKm2d
 * quantities) computed once into a DEVICE buffer (*geometry, 600 bytes per
 * cell), for fvc_cell_mesh.geometry.  It depends only on coor, ix and
 * nelcon, which must hold their values when it is called (it runs on the
 * default stream and waits for the device).  Free it with
 * fvc_cells_geometry_destroy. */
int32_t fvc_cells_geometry_create(const fvc_cell_mesh *m, void **geometry);
int32_t fvc_cells_geometry_destroy(void *geometry);

/* Green-Gauss cell gradient over the polygon of neighbour / ghost-cell
 * centroids (gform, src/Pform.f:466-646).  kind 1: velocity component comp
 * (1 or 2) with the ghost rules of src/CellibSimple.f:655-669; kind 2:
 * pressure-like field with those of src/CellibPressure.f:449-462, which
 * extrapolate with the cell's previous gradient: grad(2,numel) is read and
 * overwritten; kind 3: the ideal-gas pressure rules of src/CellibPressure.f:
 * 115-129 (comp 2: p', a prescribed-pressure face's ghost is 0; comp 3: p,
 * the ghost is sedge(3)).  FVC_ERR_UNSUPPORTED for a velocity boundary code outside
 * 0..4 (the reference leaves that ghost value undefined). */
int32_t fvc_cells_gradient(const fvc_cell_mesh *m, int32_t kind, int32_t comp,
                           const double *u, double *grad, void *stream);

/* Momentum equation of velocity component comp (cell_si_eb_i_ggl,
 * src/CellibSimple.f:591-940), one call of the reference's pform.
 * iws 1: assembles row num(c) of (ad, au) for matriz 1 (CSRD) or 4
 * (ELLPACK), b(num(c)) = the cell's right-hand side, iM(comp|comp+2,c),
 * d(comp,c) and rescell(c).  u: this component, u0: the pressure, w(2,*):
 * velocity, g_own / g_oth: the gradients of this / the other component,
 * gradp: the pressure gradient.  iws 3: only b(num(c)) = rho cc A/dt u
 * (second order in time with bs: 2 rho cc A/dt u - rho cc A/(2dt) u0). */
int32_t fvc_cells_momentum(const fvc_cell_mesh *m, int32_t comp, int32_t iws,
                           const double *u, const double *u0, const double *w,
                           const double *g_own, const double *g_oth,
                           const double *gradp, double dt, int32_t bs,
                           double under_u, int32_t simple_c, int32_t matriz,
                           const int32_t *ia, const int32_t *ja, double *ad,
                           double *au, double *b, double *im, double *d,
                           double *rescell, void *stream);

/* Momentum equation of the ideal-gas cell cell_si_eb_idg_ggl (src/
 * CellibSimple.f:54-377): the arguments of fvc_cells_momentum plus ro(3,
 * numel), the densities at levels n-1, n and the current iterate (used
 * where the incompressible cell takes the material's e(2)), div(numel), the
 * velocity divergence of the -2/3 mu div(w) terms, and gravity (gx, gy) for
 * the buoyancy source (ro - e(2)) g A.  There is no fixed-velocity pin
 * (pedge -2 is ignored); iws 3 takes the time levels from ro rows 1-2. */
int32_t fvc_cells_momentum_ideal_gas(const fvc_cell_mesh *m, int32_t comp,
                                     int32_t iws, const double *u,
                                     const double *u0, const double *w,
                                     const double *g_own, const double *g_oth,
                                     const double *gradp, const double *ro,
                                     const double *div, double gx, double gy,
                                     double dt, int32_t bs, double under_u,
                                     int32_t simple_c, int32_t matriz,
                                     const int32_t *ia, const int32_t *ja,
                                     double *ad, double *au, double *b,
                                     double *im, double *d, double *rescell,
                                     void *stream);

/* Pressure-correction equation with its right-hand side (cell_si_p_i_ggl
 * iws = 1, src/CellibPressure.f:477-572): coefficients, minus the face mass
 * fluxes of cellVel (src/CellibSimple.f:1947-2073; int_vel 1 linear, 2
 * Rhie-Chow, 5 Ferziger-Peric) into b(num(c)), the mass residual into
 * rescell(c).  w: the predicted velocity, d(2,*): momentum D, p: pressure,
 * gradp: its gradient. */
int32_t fvc_cells_pressure_correction(const fvc_cell_mesh *m, const double *w,
                                      const double *d, const double *p,
                                      const double *gradp, int32_t int_vel,
                                      int32_t matriz, const int32_t *ia,
                                      const int32_t *ja, double *ad, double *au,
                                      double *b, double *rescell, void *stream);

/* Pressure correction of the ideal-gas cell cell_si_p_idg_ggl iws = 1
 * (src/CellibPressure.f:43-246): as fvc_cells_pressure_correction with face
 * densities interpolated from ro(3,numel) (row 3, the current iterate),
 * prescribed-pressure faces (code 3) weighted by D and by the outflow /
 * backflow mass flux, no flux term for code 4, the mass storage term
 * -A (ro3 - ro2)/dt (with bs: -A (1.5 ro3 - 2 ro2 + 0.5 ro1)/dt), and
 * rescell(c) = |b(num(c))|. */
int32_t fvc_cells_pressure_correction_ideal_gas(const fvc_cell_mesh *m,
                                                const double *w, const double *d,
                                                const double *p, const double *gradp,
                                                const double *ro, int32_t int_vel,
                                                double dt, int32_t bs, int32_t matriz,
                                                const int32_t *ia, const int32_t *ja,
                                                double *ad, double *au, double *b,
                                                double *rescell, void *stream);

/* EnthalpyForTemp (src/IdealGas.f:20-50): to_temperature != 0: t = tref +
 * h/cp; else h = cp (t - tref).  The reference takes cp = e(4,1) and tref =
 * e(5,1) of material 1. */
int32_t fvc_cells_enthalpy_temperature(int32_t numel, double *h, double *t,
                                       double cp, double tref,
                                       int32_t to_temperature, void *stream);

/* idealGas (src/IdealGas.f:66-91): row `row` (1..3) of ro(3,numel) relaxed
 * toward the density of air P M/(R T): ro = (1 - under_ro) ro + under_ro
 * P M/(R T), P = 101325 Pa x pressure_ratio (cPc0/cPc of a closed domain;
 * 1 otherwise), T = temp + 273.15 when celsius. */
int32_t fvc_cells_ideal_gas_density(int32_t numel, double *ro,
                                    const double *temp, int32_t celsius,
                                    int32_t row, double pressure_ratio,
                                    double under_ro, void *stream);

/* simpleUpdate (src/Simple.f:871-910): w = u - d grad p', p += under_pc p'. */
int32_t fvc_cells_simple_update(int32_t numel, double *w, double *p,
                                const double *u1, const double *u2,
                                const double *pc, const double *gradpc,
                                const double *d, double under_pc, void *stream);

/* divergente (src/Simple.f:1070-1078): div = du1/dx + du2/dy. */
int32_t fvc_cells_divergence(int32_t numel, double *div, const double *gu1,
                             const double *gu2, void *stream);

/* Energy / transported-scalar cells of src/CellibTrans.f, one call of the
 * reference's pform (iws 1, 4) for the scalar u.  lib 3: the ideal-gas
 * enthalpy cell cell_e_eb_idg_ggl (:39-349; material k(3) conductivity,
 * k(4) specific heat, k(5) reference temperature); lib 4: the transport
 * cell cell_t_eb_ggl (:390-655).  pedge(nshared+1,numel) and
 * sedge(nshared+1,numel) are the scalar's boundary codes and values (0 flux,
 * 1 prescribed value, 2 inflow/outflow, 4 outflow; face nshared+1 a volume
 * source when its code is nonzero); m->pedge and m->sedge are not used.
 * ro(3,numel): density at levels n-1, n and the current iterate; w(2,*):
 * velocity; grad(2,*): the scalar's gradient.  iws 1: row num(c) of
 * (ad, au) for matriz 1 (CSRD) or 4 (ELLPACK), b(num(c)) and rescell(c);
 * iws 4: b(num(c)) = the time term ro cc A/dt u (second order with bs:
 * 2 ro(2) cc A/dt u - ro(1) cc A/(2dt) u0) plus the volume source.  As in
 * the reference, lib 3 truncates the boundary enthalpy cEsp (T - tRef) and
 * lib 4 the inflow density k(2) to integers. */
int32_t fvc_cells_energy(const fvc_cell_mesh *m, int32_t lib, int32_t iws,
                         const int32_t *pedge, const double *sedge,
                         const double *u, const double *u0, const double *ro,
                         const double *w, const double *grad, double dt,
                         int32_t bs, int32_t matriz, const int32_t *ia,
                         const int32_t *ja, double *ad, double *au, double *b,
                         double *rescell, void *stream);

/* Green-Gauss gradient of the scalar (gform with lib 3 or 4, src/Pform.f:
 * 466-646): ghost values from the rules of src/CellibTrans.f:131-144 (lib
 * 3: the inflow enthalpy, else extrapolation with the cell's previous
 * gradient, so grad(2,numel) is read and overwritten) and :460-464 (lib 4:
 * 2 sedge - u at inflow faces, else u). */
int32_t fvc_cells_energy_gradient(const fvc_cell_mesh *m, int32_t lib,
                                  const int32_t *pedge, const double *sedge,
                                  const double *u, double *grad, void *stream);

/* getRes (src/Solver.f:368-391): to_equations != 0: x(num(c)) = u(c);
 * else u(c) = x(num(c)). */
int32_t fvc_getres(int32_t numel, const int32_t *num, double *u, double *x,
                   int32_t to_equations, void *stream);

/* ---- SIMPLE outer iteration on the GPU ------------------------------------
 * The isothermal incompressible SIMPLE/SIMPLEC iteration of src/Simple.f:
 * 299-660 with every field, matrix and right-hand side resident on the
 * device: per outer iteration the velocity and pressure gradients, both
 * momentum systems, their solves, the p' system, its solve, the p' gradient
 * and the update, in the reference's order and with its control flow (a
 * momentum equation whose b.b < 1e-32 is not solved; no p' solve and no
 * update when the mass residual is below 1e-32).  The linear systems go
 * through the solver of this library (fvc_solve) with the reference's
 * warm-start rules.  Only the residual norms come back to the host. */
typedef struct fvc_simple fvc_simple;

typedef struct {
  double dt;          /* time step of the time term rho cc A/dt            */
  double under_u;     /* momentum under-relaxation (underU)                 */
  double under_pc;    /* pressure under-relaxation (underPc)                */
  int32_t simple_c;   /* 1: SIMPLEC's d = A/(aP - sum aNb)                  */
  int32_t bs;         /* 1: second-order backward time term                 */
  int32_t int_vel;    /* face velocity interpolation (1, 2, 5)             */
  int32_t matriz_u;   /* momentum storage: 4 ELLPACK (reference) or 1 CSRD  */
  int32_t code_u;     /* momentum solver: 2 BiCGSTAB (reference), 3 GMRES   */
  double tol_u;
  int32_t matriz_pc;  /* p' storage: 1 CSRD (reference) or 4 ELLPACK        */
  int32_t code_pc;    /* p' solver: 1 PCG (reference), 2, 3                 */
  double tol_pc;
  int32_t maxit;      /* per linear solve                                   */
  int32_t precision;  /* FVC_PREC_FP64 or FVC_PREC_MIXED for the solves     */
  int32_t precision_u; /* -1: as precision; else FVC_PREC_* for the momentum
                          and energy solves only (p' keeps precision)       */
} fvc_simple_opts;

/* Defaults: dt 1e10 (steady), underU 0.7, underPc 0.3, SIMPLE, intVel 5,
 * momentum ELLPACK + BiCGSTAB, p' CSRD + PCG, tolerances 1e-8, maxit 50000,
 * FP64 solves. */
void fvc_simple_opts_default(fvc_simple_opts *o);

/* Uploads a mesh (HOST arrays in the layouts of fvc_cell_mesh; num is the
 * equation numbering, e.g. fvc_mesh_rcm) and builds the momentum and p'
 * structures.  Fields start at rest (w = 0, p = 0) and the time term is
 * formed from them (call fvc_simple_time_step to start a new time step). */
int32_t fvc_simple_create(fvc_simple **s, int32_t device, int32_t numel,
                          int32_t nnode, int32_t nshared, int32_t nmat,
                          const double *coor, const int32_t *ix,
                          const int32_t *nelcon, const int32_t *num,
                          const int32_t *pedge, const double *sedge,
                          const double *e, const fvc_simple_opts *opts);

/* Runs nit outer iterations.  res (host, 3*nit, may be NULL) receives the
 * reference's cell-residual norms (u1, u2, p') of each iteration; its
 * (host, 3*nit, may be NULL) the linear-solver iterations (0: not solved). */
int32_t fvc_simple_iterate(fvc_simple *s, int32_t nit, double *res, int32_t *its);

/* on = 1: later fvc_simple_iterate / fvc_simple_iterate_energy calls run
 * each outer iteration as one CUDA graph launch.  The graph is captured at
 * the first such call (and again after fvc_simple_energy).  The reference's
 * host tests before each solve (a norm of at least 1e-32,
 * src/Simple.f:445-446,475-476,578-579,680-681) become conditional graph nodes
 * whose values are set on the device.  A batch of up to 256 iterations then
 * needs one host synchronisation.  The kernels, their order, and so the
 * results, the residual norms and the iteration counts are those of the
 * uncaptured loop.  A failed solve stops the solves of the rest of the
 * batch; the call returns its status with the fields as the failing
 * iteration left them, as the uncaptured loop does.  on = 0 returns to
 * individual launches.  No counterpart in the reference, whose outer loop
 * runs on the host. */
int32_t fvc_simple_set_graph(fvc_simple *s, int32_t on);

/* Starts a new time step: w0 = w and the time term from the current fields
 * (src/Simple.f:229-266). */
int32_t fvc_simple_time_step(fvc_simple *s);

/* Switches the loop to the ideal-gas iteration with the energy equation
 * (materials of type 53/55; src/Simple.f with sEnergy): momentum
 * cell_si_eb_idg_ggl with buoyancy from gravity (gx, gy), p' cell_si_p_idg_ggl,
 * then the enthalpy cell_e_eb_idg_ggl (CSRD, BiCGSTAB at tol_u) with
 * pedge_e / sedge_e (HOST, nshared+1 per cell: 0 flux, 1 temperature,
 * 2 inflow, 4 outflow; face nshared+1 a volume source), the temperature from
 * the enthalpy and the current density level from the ideal-gas law of
 * air.  Starts as src/Main.f:815-837 does: temperature t0 everywhere, the
 * enthalpy cp (t0 - tRef) with cp = e(4,1), tRef = e(5,1), all three
 * density levels from the ideal-gas law, and the time terms of a first
 * step.  The domain is open (the closed-cavity pressure rescaling is not
 * applied).  fvc_simple_time_step then shifts the density levels
 * (massUpdate) before forming the new time terms. */
int32_t fvc_simple_energy(fvc_simple *s, const int32_t *pedge_e,
                          const double *sedge_e, double gx, double gy,
                          double t0);

/* As fvc_simple_iterate for a loop switched by fvc_simple_energy; res and
 * its take 4 values per iteration: u1, u2, p', enthalpy. */
int32_t fvc_simple_iterate_energy(fvc_simple *s, int32_t nit, double *res,
                                  int32_t *its);

/* Host copies of the temperature, enthalpy (numel) and densities (3,numel)
 * of a loop switched by fvc_simple_energy; any may be NULL. */
int32_t fvc_simple_energy_fields(const fvc_simple *s, double *temp, double *en,
                                 double *ro);

/* The state a restart needs, as the reference's saveSimple writes it
 * (src/Simple.f:1307-1626): w and w0 (2,numel), p, and with the energy
 * equation en, en0 (numel) and ro (3,numel).  HOST arrays, any may be NULL;
 * en/en0/ro need a loop switched by fvc_simple_energy.  fvc_simple_set_state
 * uploads the given arrays and then starts a step from them, as the first
 * simple macro after the reference's load does: the time terms from w, w0
 * (and en, en0, ro), then w0 = w (and en0 = en); the temperature follows
 * from en. */
/* The system the last outer iteration solved (or would have solved) for
 * which = 1 u1, 2 u2, 3 p', 4 the enthalpy (a loop switched by
 * fvc_simple_energy): HOST copies, in equation order, of the diagonal ad
 * (numel), the off-diagonal values au (*nja entries) and the right-hand
 * side b (numel, the time term included), as the reference passes them to
 * `solver` (src/Simple.f:488-489,499-500,590-591,693-694).  The structure is
 * fvc_mesh_datastruc's for the system's matriz (matriz_u, matriz_pc, 1 for
 * the enthalpy).  Any pointer may be NULL; call with au NULL first to learn
 * *nja. */
int32_t fvc_simple_system(const fvc_simple *s, int32_t which, double *ad,
                          double *au, double *b, int64_t *nja);

int32_t fvc_simple_get_state(const fvc_simple *s, double *w, double *w0,
                             double *p, double *en, double *en0, double *ro);
int32_t fvc_simple_set_state(fvc_simple *s, const double *w, const double *w0,
                             const double *p, const double *en,
                             const double *en0, const double *ro);

/* Host copies of the velocity w(2,numel) and pressure p(numel); either may
 * be NULL.  fvc_simple_set_fields uploads them (e.g. to restart). */
int32_t fvc_simple_fields(const fvc_simple *s, double *w, double *p);
int32_t fvc_simple_set_fields(fvc_simple *s, const double *w, const double *p);

int32_t fvc_simple_destroy(fvc_simple *s);

/* ---- many SIMPLE cases together ------------------------------------------ */
/* No single counterpart in the reference, which runs one case per process
 * (src/Simple.f:317-801 per case).  The outer iterations of ncases
 * independent loops (each an fvc_simple from fvc_simple_create, with
 * fvc_simple_energy for all of them or for none; CSRD systems, matriz_u =
 * matriz_pc = 1; one device; one maxit), with the linear solves of every
 * stage in one persistent launch: all u1 and u2 systems, then all p'
 * systems, then all enthalpy systems, each system with its own convergence
 * test, tolerance (its case's tol_u / tol_pc), method (code_u / code_pc;
 * BiCGSTAB for the enthalpy) and status.  precision (the p' systems) and
 * precision_u (u, v and the enthalpy; < 0: as precision): FVC_PREC_FP64 or
 * FVC_PREC_MIXED (FP32 iterations, FP64 refinement to the same tolerances
 * on ||b - Ax||2 / ||b||2).  A mixed BiCGSTAB whose FP32 sweeps stall is
 * finished in FP64 from its FP32 iterate inside the same graph, as fvc_solve
 * finishes one (a second, FP64 launch of the stage in which every other
 * system is masked out).  The reference's tests before a
 * solve skip that system inside the launch (a per-system mask), and the work
 * after a skipped p' or enthalpy solve is skipped with it.  Each outer
 * iteration of all cases is one CUDA graph launch (captured at the first
 * call, and again after the first outer iteration with each system's
 * iteration count as its share of the launch's blocks).  The batch borrows
 * the cases, which must outlive it; their fields are those of the loops
 * (fvc_simple_fields etc.).  ncases is limited by the co-resident blocks of
 * one launch (1216 on this GPU at 128 threads: 608 cases). */
typedef struct fvc_simple_batch fvc_simple_batch;
int32_t fvc_simple_batch_create(fvc_simple_batch **out, int32_t ncases,
                                fvc_simple *const *cases, int32_t precision,
                                int32_t precision_u);
/* nit outer iterations of every case.  res (may be NULL) receives, per
 * iteration and case, the norms fvc_simple_iterate (3: u1, u2, p') or
 * fvc_simple_iterate_energy (4: and the enthalpy) return, at
 * res[(it * ncases + case) * nres + k]; its likewise the solver iterations
 * (FP32 ones for mixed, 0 where a solve was skipped).  A failed solve ends
 * the call with its status after the outer iteration it failed in. */
int32_t fvc_simple_batch_iterate(fvc_simple_batch *b, int32_t nit, double *res,
                                 int32_t *its);
int32_t fvc_simple_batch_destroy(fvc_simple_batch *b);

#ifdef __cplusplus
}
#endif
#endif
