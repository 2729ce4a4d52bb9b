// fvc_simple_driver.cu -- the isothermal SIMPLE outer iteration of
// src/Simple.f:299-660 with all fields, matrices and right-hand sides on
// the GPU.  Each outer iteration runs, in the reference's order: guess
// (u = w), the velocity gradients, divergente, the pressure gradient, both
// momentum systems (+ the time-term right-hand side b0, and the cell
// residuals + getRes(b0)), their solves, updateVel, the p' system, its
// solve, the p' gradient and simpleUpdate.  The cell kernels are those of
// fvc_simple.cu; the solves go through fvc_solve on two solver contexts
// (momentum, p'), whose values are refreshed from the device each time.
// Only the few norms that steer the reference's control flow cross to the
// host.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include <cuda_runtime.h>

#include "fvc_internal.h"

namespace fvc {
namespace {

constexpr int kT = 256;

__global__ void split_w(int n, const double *w, double *u1, double *u2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    u1[i] = w[2 * (size_t)i];
    u2[i] = w[2 * (size_t)i + 1];
  }
}

__global__ void join_w(int n, double *w, const double *u1, const double *u2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    w[2 * (size_t)i] = u1[i];
    w[2 * (size_t)i + 1] = u2[i];
  }
}

// asumb(b, b0) and rc(c) += b0(num(c)) (Simple.f:423-425)
__global__ void add_time_term(int n, const int32_t *num, double *b, const double *b0,
                              double *rc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    b[i] = b[i] + b0[i];
    rc[i] = rc[i] + b0[num[i] - 1];
  }
}

// out[k] = x_k . x_k for up to 3 vectors, one block each, fixed order
__global__ void self_dots(int n, const double *a, const double *b, const double *c, double *out) {
  __shared__ double red[kT];
  const double *x = (blockIdx.x == 0) ? a : (blockIdx.x == 1) ? b : c;
  double t = 0.0;
  for (int i = threadIdx.x; i < n; i += kT) t = fma(x[i], x[i], t);
  red[threadIdx.x] = t;
  __syncthreads();
  for (int s = kT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

inline int g(int n) { return (n + kT - 1) / kT; }

// One outer iteration of the captured loop (fvc_simple_set_graph): the
// norms that steer it and what each solve (u1, u2, p', energy) returned.
struct SimpleRec {
  double dots[8];   // |b1|^2 |b2|^2, |rc1|^2 |rc2|^2 |rcp|^2, |be|^2 |rce|^2
  int32_t st[4][4]; // status, iterations, inner iterations, timeout flag
  int32_t ran[4];   // the solve ran
  int32_t ok[4];    // ... and ended with FVC_OK
};
constexpr int kRecMax = 256;  // outer iterations per batch of graph launches

// ctr[0]: the record of the running iteration; ctr[1]: a solve failed
__global__ void rec_dots(const int32_t *ctr, SimpleRec *rec, const double *dots, int off,
                         int k) {
  SimpleRec &r = rec[ctr[0]];
  for (int i = 0; i < k; ++i) r.dots[off + i] = dots[i];
}

// The reference's test before a solve (the norm, or its square root, at
// least 1e-32), and no solve failed before it in this batch.
__global__ void set_run(cudaGraphConditionalHandle h, const int32_t *ctr, SimpleRec *rec,
                        int dot, int use_sqrt, int sys) {
  SimpleRec &r = rec[ctr[0]];
  const double v = use_sqrt ? sqrt(r.dots[dot]) : r.dots[dot];
  const int run = (v >= 1.0e-32 && ctr[1] == 0) ? 1 : 0;
  r.ran[sys] = run;
  cudaGraphSetConditional(h, (unsigned)run);
}

// After a solve: its status into the record; a failure stops the solves of
// the rest of the batch, as the uncaptured loop returns at the first one.
__global__ void set_ok(cudaGraphConditionalHandle h, int32_t *ctr, SimpleRec *rec,
                       const int32_t *st, int sys) {
  SimpleRec &r = rec[ctr[0]];
  int ok = 0;
  if (r.ran[sys]) {
    for (int k = 0; k < 4; ++k) r.st[sys][k] = st[k];
    ok = (st[0] == 0) ? 1 : 0;
    if (!ok) ctr[1] = 1;
  }
  r.ok[sys] = ok;
  cudaGraphSetConditional(h, (unsigned)ok);
}

__global__ void next_rec(int32_t *ctr) { ctr[0] += 1; }

}  // namespace
}  // namespace fvc

struct fvc_simple {
  int device = 0;
  cudaStream_t stream = nullptr;
  fvc_simple_opts o{};
  int numel = 0, nshared = 0, nnode = 0, nmat = 0;
  fvc_cell_mesh m{};
  // device mesh storage
  double *coor = nullptr, *sedge = nullptr, *e = nullptr;
  int32_t *ix = nullptr, *nelcon = nullptr, *num = nullptr, *pedge = nullptr;
  // structures (device copies for the cell scatter)
  int32_t *ia_u = nullptr, *ja_u = nullptr, *ia_pc = nullptr, *ja_pc = nullptr;
  size_t nja_u = 0, nja_pc = 0;
  fvc_context *ctx_u = nullptr, *ctx_pc = nullptr;
  // fields and systems
  double *w = nullptr, *w0 = nullptr, *p = nullptr, *pc = nullptr, *u1 = nullptr, *u2 = nullptr;
  double *gu1 = nullptr, *gu2 = nullptr, *gp = nullptr, *gpc = nullptr, *d = nullptr;
  double *im = nullptr, *div = nullptr, *wp = nullptr;
  double *ad1 = nullptr, *au1 = nullptr, *b1 = nullptr, *ad2 = nullptr, *au2 = nullptr,
         *b2 = nullptr;
  double *b10 = nullptr, *b20 = nullptr, *adp = nullptr, *aup = nullptr, *bp = nullptr;
  double *rc1 = nullptr, *rc2 = nullptr, *rcp = nullptr, *xe = nullptr, *dots = nullptr;
  double *h_dots = nullptr;  // pinned
  // ideal gas with the energy equation (fvc_simple_energy)
  bool gas = false;
  double grav[2] = {0.0, 0.0}, cp = 0.0, tref = 0.0;
  int32_t *pedge_e = nullptr, *ia_e = nullptr, *ja_e = nullptr;
  double *sedge_e = nullptr;
  size_t nja_e = 0;
  fvc_context *ctx_e = nullptr;
  double *ro = nullptr, *en = nullptr, *en0 = nullptr, *temp = nullptr, *ge = nullptr;
  double *ade = nullptr, *aue = nullptr, *be = nullptr, *be0 = nullptr, *rce = nullptr;
  std::vector<int32_t> ident;
  std::vector<void *> owned;
  int32_t *d_err = nullptr, *h_err = nullptr;  // gradient: unsupported boundary code
  // one outer iteration as a CUDA graph (fvc_simple_set_graph)
  bool use_graph = false, graph_gas = false;
  cudaStream_t body = nullptr;  // captures the bodies of the conditional nodes
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  fvc::SimpleRec *rec = nullptr, *h_rec = nullptr;
  int32_t *gctr = nullptr, *st_tmp = nullptr;
  int64_t launches_top = 0, launches_run[4] = {0, 0, 0, 0}, launches_ok[4] = {0, 0, 0, 0};
};

namespace {

template <typename T>
int32_t dalloc(fvc_simple *s, T *&ptr, size_t n) {
  if (cudaMalloc(&ptr, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) return FVC_ERR_CUDA;
  s->owned.push_back(ptr);
  return cudaMemsetAsync(ptr, 0, sizeof(T) * std::max<size_t>(n, 1), s->stream) == cudaSuccess
             ? FVC_OK
             : FVC_ERR_CUDA;
}

template <typename T>
int32_t dcopy(fvc_simple *s, T *&ptr, const T *h, size_t n) {
  int32_t rc = dalloc(s, ptr, n);
  if (rc != FVC_OK) return rc;
  return cudaMemcpyAsync(ptr, h, sizeof(T) * n, cudaMemcpyHostToDevice, s->stream) == cudaSuccess
             ? FVC_OK
             : FVC_ERR_CUDA;
}

void release(fvc_simple *s) {
  if (s->ctx_u) fvc_context_destroy(s->ctx_u);
  if (s->ctx_pc) fvc_context_destroy(s->ctx_pc);
  if (s->ctx_e) fvc_context_destroy(s->ctx_e);
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  if (s->graph) cudaGraphDestroy(s->graph);
  if (s->body) cudaStreamDestroy(s->body);
  for (void *ptr : s->owned) cudaFree(ptr);
  if (s->h_dots) cudaFreeHost(s->h_dots);
  if (s->h_err) cudaFreeHost(s->h_err);
  if (s->h_rec) cudaFreeHost(s->h_rec);
  if (s->stream) cudaStreamDestroy(s->stream);
}

// one system's structure on the host, then a solver context holding it
int32_t make_system(fvc_simple *s, const std::vector<int32_t> &ident, int matriz,
                    fvc_context **ctx, int32_t **d_ia, int32_t **d_ja, size_t *nja) {
  const int neq = s->numel;
  std::vector<int32_t> ia(matriz == 4 ? 2 : neq + 1);
  int32_t nad = 0;
  int64_t len = 0;
  int32_t rc = fvc_mesh_datastruc(ident.data(), neq, s->nshared, matriz, 1, ia.data(), nullptr,
                                  &nad, &len);
  if (rc != FVC_OK) return rc;
  std::vector<int32_t> ja((size_t)std::max<int64_t>(len, 1));
  rc = fvc_mesh_datastruc(ident.data(), neq, s->nshared, matriz, 1, ia.data(), ja.data(), &nad,
                          &len);
  if (rc != FVC_OK) return rc;
  *nja = (size_t)len;
  if ((rc = dcopy(s, *d_ia, ia.data(), ia.size())) != FVC_OK) return rc;
  if ((rc = dcopy(s, *d_ja, ja.data(), ja.size())) != FVC_OK) return rc;
  if ((rc = fvc_context_create(ctx, s->device)) != FVC_OK) return rc;
  fvc_context_set_stream(*ctx, s->stream);
  // structure with placeholder values (unit diagonal); real values arrive
  // from the device before every solve
  std::vector<double> ad(neq, 1.0), au((size_t)std::max<int64_t>(len, 1), 0.0);
  return fvc_matrix_set(*ctx, matriz, 1, neq, nad, ad.data(), au.data(), au.data(), ia.data(),
                        ja.data());
}

// start of a time step with the ideal gas (src/Simple.f:229-300): momentum
// time terms from the densities of levels n-1 and n, w0 = w, the enthalpy's
// time term and volume source, en0 = en
int32_t time_term_gas(fvc_simple *s) {
  const int n = s->numel;
  fvc::split_w<<<fvc::g(n), fvc::kT, 0, s->stream>>>(n, s->w, s->u1, s->u2);
  fvc::count_launch();
  double *u0a = s->wp, *u0b = s->xe;  // the previous level (read only with bs)
  fvc::split_w<<<fvc::g(n), fvc::kT, 0, s->stream>>>(n, s->w0, u0a, u0b);
  fvc::count_launch();
  const int mu = s->o.matriz_u;
  int32_t rc;
  for (int comp = 1; comp <= 2; ++comp) {
    rc = fvc_cells_momentum_ideal_gas(&s->m, comp, 3, comp == 1 ? s->u1 : s->u2,
                                      comp == 1 ? u0a : u0b, nullptr, nullptr, nullptr, nullptr,
                                      s->ro, nullptr, s->grav[0], s->grav[1], s->o.dt, s->o.bs,
                                      s->o.under_u, s->o.simple_c, mu, s->ia_u, s->ja_u, nullptr,
                                      nullptr, comp == 1 ? s->b10 : s->b20, nullptr, nullptr,
                                      nullptr, s->stream);
    if (rc != FVC_OK) return rc;
  }
  if (cudaMemcpyAsync(s->w0, s->w, sizeof(double) * 2 * n, cudaMemcpyDeviceToDevice,
                      s->stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  rc = fvc_cells_energy(&s->m, 3, 4, s->pedge_e, s->sedge_e, s->en, s->en0, s->ro, nullptr,
                        nullptr, s->o.dt, s->o.bs, 1, s->ia_e, s->ja_e, nullptr, nullptr, s->be0,
                        nullptr, s->stream);
  if (rc != FVC_OK) return rc;
  return cudaMemcpyAsync(s->en0, s->en, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                         s->stream) == cudaSuccess
             ? FVC_OK
             : FVC_ERR_CUDA;
}

// massUpdate (src/Simple.f:1041-1050): ro(1) = ro(2), ro(2) = ro(3)
__global__ void mass_update(int n, double *ro) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  ro[3 * (size_t)i] = ro[3 * (size_t)i + 1];
  ro[3 * (size_t)i + 1] = ro[3 * (size_t)i + 2];
}

__global__ void fill(int n, double *x, double v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

int32_t time_term(fvc_simple *s) {
  const int n = s->numel;
  fvc::split_w<<<fvc::g(n), fvc::kT, 0, s->stream>>>(n, s->w, s->u1, s->u2);
  fvc::count_launch();
  double *u0a = nullptr, *u0b = nullptr;
  if (s->o.bs) {  // u0: the previous time level
    u0a = s->wp;
    u0b = s->xe;
    fvc::split_w<<<fvc::g(n), fvc::kT, 0, s->stream>>>(n, s->w0, u0a, u0b);
    fvc::count_launch();
  }
  const int mu = s->o.matriz_u;
  int32_t rc = fvc_cells_momentum(&s->m, 1, 3, s->u1, u0a, nullptr, nullptr, nullptr, nullptr,
                                  s->o.dt, s->o.bs, s->o.under_u, s->o.simple_c, mu, s->ia_u,
                                  s->ja_u, nullptr, nullptr, s->b10, nullptr, nullptr, nullptr,
                                  s->stream);
  if (rc != FVC_OK) return rc;
  return fvc_cells_momentum(&s->m, 2, 3, s->u2, u0b, nullptr, nullptr, nullptr, nullptr,
                            s->o.dt, s->o.bs, s->o.under_u, s->o.simple_c, mu, s->ia_u,
                            s->ja_u, nullptr, nullptr, s->b20, nullptr, nullptr, nullptr,
                            s->stream);
}

// p' (ctx_pc) takes precision; momentum and energy precision_u when set
fvc_opts solve_opts(const fvc_simple *s, const fvc_context *ctx) {
  fvc_opts o;
  fvc_opts_default(&o);
  o.precision = (ctx != s->ctx_pc && s->o.precision_u >= 0) ? s->o.precision_u : s->o.precision;
  return o;
}

// x (cells) -> equation order, solve, back to cells
int32_t solve(fvc_simple *s, fvc_context *ctx, int code, const double *ad, const double *au,
              const double *b, double *x_cells, double tol, int *its, const char *what) {
  const int n = s->numel;
  int32_t rc = fvc_getres(n, s->num, x_cells, s->xe, 1, s->stream);
  if (rc != FVC_OK) return rc;
  if ((rc = fvc_matrix_update_values_async(ctx, ad, au, au)) != FVC_OK) return rc;
  const fvc_opts o = solve_opts(s, ctx);
  fvc_stats st;
  rc = fvc_solve(ctx, code, b, s->xe, tol, s->o.maxit, &o, &st);
  if (its) *its = st.iterations;
  if (rc != FVC_OK) {
    // the reference prints the failing solve before it stops
    fprintf(stderr, "fvcgpu: SIMPLE %s solve (code %d, %s) ended with status %d after %d "
                    "iterations\n", what, code, o.precision == FVC_PREC_MIXED ? "mixed" : "fp64",
            rc, st.iterations);
    return rc;
  }
  return fvc_getres(n, s->num, x_cells, s->xe, 0, s->stream);
}

}  // namespace

extern "C" {

void fvc_simple_opts_default(fvc_simple_opts *o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->dt = 1.0e10;
  o->under_u = 0.7;
  o->under_pc = 0.3;
  o->int_vel = 5;
  o->matriz_u = 4;
  o->code_u = 2;
  o->tol_u = 1.0e-8;
  o->matriz_pc = 1;
  o->code_pc = 1;
  o->tol_pc = 1.0e-8;
  o->maxit = 50000;
  o->precision = FVC_PREC_FP64;
  o->precision_u = -1;
}

int32_t fvc_simple_create(fvc_simple **out, int32_t device, int32_t numel, int32_t nnode,
                          int32_t nshared, int32_t nmat, const double *coor, const int32_t *ix,
                          const int32_t *nelcon, const int32_t *num, const int32_t *pedge,
                          const double *sedge, const double *e, const fvc_simple_opts *opts) {
  if (!out) return FVC_ERR_ARG;
  *out = nullptr;
  if (numel <= 0 || nnode <= 0 || nmat <= 0 || (nshared != 3 && nshared != 4) || !coor || !ix ||
      !nelcon || !num || !pedge || !sedge || !e)
    return FVC_ERR_ARG;
  fvc_simple_opts o;
  if (opts)
    o = *opts;
  else
    fvc_simple_opts_default(&o);
  if ((o.matriz_u != 1 && o.matriz_u != 4) || (o.matriz_pc != 1 && o.matriz_pc != 4) ||
      o.code_u < 1 || o.code_u > 3 || o.code_pc < 1 || o.code_pc > 3 || o.dt == 0.0 ||
      o.maxit <= 0)
    return FVC_ERR_ARG;
  if (o.int_vel != 1 && o.int_vel != 2 && o.int_vel != 5) return FVC_ERR_UNSUPPORTED;
  fvc_simple *s = new (std::nothrow) fvc_simple();
  if (!s) return FVC_ERR_ARG;
  s->device = device;
  s->o = o;
  s->numel = numel;
  s->nshared = nshared;
  s->nnode = nnode;
  s->nmat = nmat;
  int32_t rc = FVC_OK;
  auto fail = [&](int32_t r) {
    release(s);
    delete s;
    return r;
  };
  if (cudaSetDevice(device) != cudaSuccess) return fail(FVC_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(FVC_ERR_CUDA);
  const size_t n = numel, ld = nshared + 1;
  if ((rc = dcopy(s, s->coor, coor, 2 * (size_t)nnode)) != FVC_OK ||
      (rc = dcopy(s, s->ix, ix, ld * n)) != FVC_OK ||
      (rc = dcopy(s, s->nelcon, nelcon, (size_t)nshared * n)) != FVC_OK ||
      (rc = dcopy(s, s->num, num, n)) != FVC_OK ||
      (rc = dcopy(s, s->pedge, pedge, ld * n)) != FVC_OK ||
      (rc = dcopy(s, s->sedge, sedge, 3 * ld * n)) != FVC_OK ||
      (rc = dcopy(s, s->e, e, 10 * (size_t)nmat)) != FVC_OK)
    return fail(rc);
  s->m.numel = numel;
  s->m.nshared = nshared;
  s->m.nnode = nnode;
  s->m.nmat = nmat;
  s->m.coor = s->coor;
  s->m.ix = s->ix;
  s->m.nelcon = s->nelcon;
  s->m.num = s->num;
  s->m.pedge = s->pedge;
  s->m.sedge = s->sedge;
  s->m.e = s->e;
  std::vector<int32_t> &ident = s->ident;
  ident.resize((size_t)nshared * n);
  if ((rc = fvc_mesh_numeq(num, nelcon, numel, nshared, ident.data())) != FVC_OK) return fail(rc);
  s->cp = e[3];    // e(4,1), e(5,1): the reference's EnthalpyForTemp uses material 1
  s->tref = e[4];
  if ((rc = make_system(s, ident, o.matriz_u, &s->ctx_u, &s->ia_u, &s->ja_u, &s->nja_u)) !=
      FVC_OK)
    return fail(rc);
  if ((rc = make_system(s, ident, o.matriz_pc, &s->ctx_pc, &s->ia_pc, &s->ja_pc, &s->nja_pc)) !=
      FVC_OK)
    return fail(rc);
  double **vec[] = {&s->p, &s->pc, &s->u1, &s->u2, &s->div, &s->ad1, &s->b1, &s->ad2, &s->b2,
                    &s->b10, &s->b20, &s->adp, &s->bp, &s->rc1, &s->rc2, &s->rcp, &s->xe};
  for (double **v : vec)
    if ((rc = dalloc(s, *v, n)) != FVC_OK) return fail(rc);
  double **vec2[] = {&s->w, &s->w0, &s->gu1, &s->gu2, &s->gp, &s->gpc, &s->d, &s->wp};
  for (double **v : vec2)
    if ((rc = dalloc(s, *v, 2 * n)) != FVC_OK) return fail(rc);
  if ((rc = dalloc(s, s->im, 4 * n)) != FVC_OK || (rc = dalloc(s, s->au1, s->nja_u)) != FVC_OK ||
      (rc = dalloc(s, s->au2, s->nja_u)) != FVC_OK ||
      (rc = dalloc(s, s->aup, s->nja_pc)) != FVC_OK || (rc = dalloc(s, s->dots, 4)) != FVC_OK)
    return fail(rc);
  if ((rc = dalloc(s, s->d_err, 1)) != FVC_OK) return fail(rc);
  if (cudaMallocHost(&s->h_dots, 4 * sizeof(double)) != cudaSuccess ||
      cudaMallocHost(&s->h_err, sizeof(int32_t)) != cudaSuccess)
    return fail(FVC_ERR_CUDA);
  if ((rc = time_term(s)) != FVC_OK) return fail(rc);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return fail(FVC_ERR_CUDA);
  *out = s;
  return FVC_OK;
}

int32_t fvc_simple_time_step(fvc_simple *s) {
  if (!s) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  if (s->gas) {
    mass_update<<<fvc::g(s->numel), fvc::kT, 0, s->stream>>>(s->numel, s->ro);
    fvc::count_launch();
    int32_t rc = time_term_gas(s);
    if (rc != FVC_OK) return rc;
    return cudaStreamSynchronize(s->stream) == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
  }
  int32_t rc = time_term(s);
  if (rc != FVC_OK) return rc;
  if (cudaMemcpyAsync(s->w0, s->w, sizeof(double) * 2 * s->numel, cudaMemcpyDeviceToDevice,
                      s->stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  return cudaStreamSynchronize(s->stream) == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

}  // extern "C"

namespace {

// ---- stages of one outer iteration (src/Simple.f:299-710) ------------------
// Each enqueues on st and returns without waiting; the loop below (or the
// capture of a graph) reads the norms they leave in s->dots.

// guess, the gradients of u1, u2 (momentum ghost rules) and p, divergente,
// both momentum systems with the time term and cell residuals; dots =
// |b1|^2, |b2|^2
int32_t stage_momentum(fvc_simple *s, cudaStream_t st) {
  const bool gas = s->gas;
  const int n = s->numel, mu = s->o.matriz_u;
  const fvc_cell_mesh *m = &s->m;
  int32_t rc;
  fvc::split_w<<<fvc::g(n), fvc::kT, 0, st>>>(n, s->w, s->u1, s->u2);
  fvc::count_launch();
  if ((rc = fvc::cells::gradient_async(m, 1, 1, s->u1, s->gu1, s->d_err, st)) != FVC_OK ||
      (rc = fvc::cells::gradient_async(m, 1, 2, s->u2, s->gu2, s->d_err, st)) != FVC_OK)
    return rc;
  if ((rc = fvc_cells_divergence(n, s->div, s->gu1, s->gu2, st)) != FVC_OK) return rc;
  // the pressure's ghost rules: incompressible, or the ideal-gas cell's (p)
  if ((rc = fvc::cells::gradient_async(m, gas ? 3 : 2, 3, s->p, s->gp, s->d_err, st)) != FVC_OK)
    return rc;
  // momentum systems (u0 = p), time term, cell residuals
  for (int comp = 1; comp <= 2; ++comp) {
    double *u = comp == 1 ? s->u1 : s->u2, *ad = comp == 1 ? s->ad1 : s->ad2;
    double *au = comp == 1 ? s->au1 : s->au2, *b = comp == 1 ? s->b1 : s->b2;
    double *rcv = comp == 1 ? s->rc1 : s->rc2;
    const double *ga = comp == 1 ? s->gu1 : s->gu2, *gb = comp == 1 ? s->gu2 : s->gu1;
    if (gas)
      rc = fvc_cells_momentum_ideal_gas(m, comp, 1, u, s->p, s->w, ga, gb, s->gp, s->ro, s->div,
                                        s->grav[0], s->grav[1], s->o.dt, s->o.bs, s->o.under_u,
                                        s->o.simple_c, mu, s->ia_u, s->ja_u, ad, au, b, s->im,
                                        s->d, rcv, st);
    else
      rc = fvc_cells_momentum(m, comp, 1, u, s->p, s->w, ga, gb, s->gp, s->o.dt, s->o.bs,
                              s->o.under_u, s->o.simple_c, mu, s->ia_u, s->ja_u, ad, au, b, s->im,
                              s->d, rcv, st);
    if (rc != FVC_OK) return rc;
    fvc::add_time_term<<<fvc::g(n), fvc::kT, 0, st>>>(n, s->num, b, comp == 1 ? s->b10 : s->b20,
                                                      rcv);
    fvc::count_launch();
  }
  fvc::self_dots<<<2, fvc::kT, 0, st>>>(n, s->b1, s->b2, s->b2, s->dots);
  fvc::count_launch();
  return FVC_OK;
}

// updateVel, the p' system; dots = |rc1|^2, |rc2|^2, |rcp|^2
int32_t stage_pressure(fvc_simple *s, cudaStream_t st) {
  const int n = s->numel, mpc = s->o.matriz_pc;
  int32_t rc;
  fvc::join_w<<<fvc::g(n), fvc::kT, 0, st>>>(n, s->wp, s->u1, s->u2);
  fvc::count_launch();
  if (s->gas)
    rc = fvc_cells_pressure_correction_ideal_gas(&s->m, s->wp, s->d, s->p, s->gp, s->ro,
                                                 s->o.int_vel, s->o.dt, s->o.bs, mpc, s->ia_pc,
                                                 s->ja_pc, s->adp, s->aup, s->bp, s->rcp, st);
  else
    rc = fvc_cells_pressure_correction(&s->m, s->wp, s->d, s->p, s->gp, s->o.int_vel, mpc,
                                       s->ia_pc, s->ja_pc, s->adp, s->aup, s->bp, s->rcp, st);
  if (rc != FVC_OK) return rc;
  fvc::self_dots<<<3, fvc::kT, 0, st>>>(n, s->rc1, s->rc2, s->rcp, s->dots);
  fvc::count_launch();
  return FVC_OK;
}

// after the p' solve: its gradient and simpleUpdate
int32_t after_pressure(fvc_simple *s, cudaStream_t st) {
  int32_t rc = fvc::cells::gradient_async(&s->m, s->gas ? 3 : 2, 2, s->pc, s->gpc, s->d_err, st);
  if (rc != FVC_OK) return rc;
  return fvc_cells_simple_update(s->numel, s->w, s->p, s->u1, s->u2, s->pc, s->gpc, s->d,
                                 s->o.under_pc, st);
}

// the enthalpy system (src/Simple.f:647-710); dots = |be|^2, |rce|^2
int32_t stage_energy(fvc_simple *s, cudaStream_t st) {
  const int n = s->numel;
  const fvc_cell_mesh *m = &s->m;
  int32_t rc;
  if ((rc = fvc_cells_energy_gradient(m, 3, s->pedge_e, s->sedge_e, s->en, s->ge, st)) != FVC_OK)
    return rc;
  if ((rc = fvc_cells_energy(m, 3, 1, s->pedge_e, s->sedge_e, s->en, s->en, s->ro, s->w, s->ge,
                             s->o.dt, s->o.bs, 1, s->ia_e, s->ja_e, s->ade, s->aue, s->be, s->rce,
                             st)) != FVC_OK)
    return rc;
  fvc::add_time_term<<<fvc::g(n), fvc::kT, 0, st>>>(n, s->num, s->be, s->be0, s->rce);
  fvc::count_launch();
  fvc::self_dots<<<2, fvc::kT, 0, st>>>(n, s->be, s->rce, s->rce, s->dots);
  fvc::count_launch();
  return FVC_OK;
}

// after the energy solve: temperatures and the new density level
int32_t after_energy(fvc_simple *s, cudaStream_t st) {
  int32_t rc = fvc_cells_enthalpy_temperature(s->numel, s->en, s->temp, s->cp, s->tref, 1, st);
  if (rc != FVC_OK) return rc;
  return fvc_cells_ideal_gas_density(s->numel, s->ro, s->temp, 1, 3, 1.0, 1.0, st);
}

int32_t read_dots(fvc_simple *s, int k, bool err) {
  cudaMemcpyAsync(s->h_dots, s->dots, k * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
  if (err) cudaMemcpyAsync(s->h_err, s->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return FVC_ERR_CUDA;
  return (err && *s->h_err) ? FVC_ERR_UNSUPPORTED : FVC_OK;  // a velocity code outside 0..4
}

// nit outer iterations with the norms read back where the reference tests
// them; res/its get nrep entries per iteration
int32_t iterate_plain(fvc_simple *s, int32_t nit, double *res, int32_t *its, int nrep) {
  cudaStream_t st = s->stream;
  int32_t rc;
  for (int it = 0; it < nit; ++it) {
    int solver_its[4] = {0, 0, 0, 0};
    if ((rc = stage_momentum(s, st)) != FVC_OK || (rc = read_dots(s, 2, true)) != FVC_OK)
      return rc;
    const bool solve1 = s->h_dots[0] >= 1.0e-32, solve2 = s->h_dots[1] >= 1.0e-32;
    if (solve1 && (rc = solve(s, s->ctx_u, s->o.code_u, s->ad1, s->au1, s->b1, s->u1,
                              s->o.tol_u, &solver_its[0], "u1")) != FVC_OK)
      return rc;
    if (solve2 && (rc = solve(s, s->ctx_u, s->o.code_u, s->ad2, s->au2, s->b2, s->u2,
                              s->o.tol_u, &solver_its[1], "u2")) != FVC_OK)
      return rc;
    if ((rc = stage_pressure(s, st)) != FVC_OK || (rc = read_dots(s, 3, false)) != FVC_OK)
      return rc;
    const double r1 = std::sqrt(s->h_dots[0]), r2 = std::sqrt(s->h_dots[1]);
    const double rpc = std::sqrt(s->h_dots[2]);
    if (rpc >= 1.0e-32) {
      if ((rc = solve(s, s->ctx_pc, s->o.code_pc, s->adp, s->aup, s->bp, s->pc, s->o.tol_pc,
                      &solver_its[2], "p'")) != FVC_OK ||
          (rc = after_pressure(s, st)) != FVC_OK)
        return rc;
    }
    double re = 0.0;
    if (s->gas) {
      if ((rc = stage_energy(s, st)) != FVC_OK || (rc = read_dots(s, 2, false)) != FVC_OK)
        return rc;
      re = std::sqrt(s->h_dots[0]);
      if (re >= 1.0e-32) {
        re = std::sqrt(s->h_dots[1]);
        if ((rc = solve(s, s->ctx_e, 2, s->ade, s->aue, s->be, s->en, s->o.tol_u,
                        &solver_its[3], "energy")) != FVC_OK ||
            (rc = after_energy(s, st)) != FVC_OK)
          return rc;
      }
    }
    if (res) {
      res[nrep * it] = r1;
      res[nrep * it + 1] = r2;
      res[nrep * it + 2] = rpc;
      if (nrep == 4) res[4 * it + 3] = re;
    }
    if (its)
      for (int k = 0; k < nrep; ++k) its[nrep * it + k] = solver_its[k];
  }
  return cudaStreamSynchronize(st) == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

// ---- one outer iteration as a CUDA graph -----------------------------------
// The stages above, captured once.  The reference's host tests before each
// solve become conditional (IF) nodes whose values kernels set from the
// norms on the device, so one graph launch runs a whole outer iteration and
// a batch of launches needs one host synchronisation at its end.

// A failed CUDA call while the graph is captured: names the call
bool cap_ok(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  fprintf(stderr, "fvcgpu: graph capture: %s: %s\n", what, cudaGetErrorString(e));
  return false;
}

// Adds an IF node on h to the capture running on s->stream and captures
// body(stream) into the node's body graph on s->body.
template <typename F>
int32_t cap_if(fvc_simple *s, cudaGraphConditionalHandle h, int64_t *launches, F body) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  const cudaGraphEdgeData *ed = nullptr;
  size_t nd = 0;
  if (!cap_ok(cudaStreamGetCaptureInfo(s->stream, &cs, nullptr, &g, &deps, &ed, &nd),
              "cudaStreamGetCaptureInfo"))
    return FVC_ERR_CUDA;
  if (cs != cudaStreamCaptureStatusActive) {
    fprintf(stderr, "fvcgpu: graph capture: the capture was invalidated (status %d)\n",
            (int)cs);
    return FVC_ERR_CUDA;
  }
  cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeIf;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if (!cap_ok(cudaGraphAddNode(&node, g, deps, ed, nd, &p), "cudaGraphAddNode (IF)") ||
      !cap_ok(cudaStreamUpdateCaptureDependencies(s->stream, &node, nullptr, 1,
                                                  cudaStreamSetCaptureDependencies),
              "cudaStreamUpdateCaptureDependencies"))
    return FVC_ERR_CUDA;
  if (!cap_ok(cudaStreamBeginCaptureToGraph(s->body, p.conditional.phGraph_out[0], nullptr,
                                            nullptr, 0, cudaStreamCaptureModeRelaxed),
              "cudaStreamBeginCaptureToGraph"))
    return FVC_ERR_CUDA;
  const int64_t l0 = fvc_kernel_launches();
  const int32_t rc = body(s->body);
  *launches = fvc_kernel_launches() - l0;
  cudaGraph_t out = nullptr;  // the body graph itself, owned by the node
  const bool ended = cap_ok(cudaStreamEndCapture(s->body, &out), "cudaStreamEndCapture (body)");
  if (rc != FVC_OK) {
    fprintf(stderr, "fvcgpu: graph capture: a body enqueue returned status %d\n", rc);
    return rc;
  }
  return ended ? FVC_OK : FVC_ERR_CUDA;
}

// One system's solve inside the captured iteration: IF(run) { x to
// equation order, the values, the solve, its status }, the status into the
// record, IF(ok) { x back to the cells, then after(stream) }.
template <typename F>
int32_t cap_solve(fvc_simple *s, int sys, fvc_context *ctx, int code, const double *ad,
                  const double *au, const double *b, double *x_cells, double tol,
                  cudaGraphConditionalHandle hrun, cudaGraphConditionalHandle hok, F after) {
  const int n = s->numel;
  const fvc_opts o = solve_opts(s, ctx);
  int32_t *stp = s->st_tmp + 4 * sys;
  int32_t rc = cap_if(s, hrun, &s->launches_run[sys], [&](cudaStream_t bs) {
    int32_t r = fvc_getres(n, s->num, x_cells, s->xe, 1, bs);
    if (r != FVC_OK) return r;
    fvc_context_set_stream(ctx, bs);
    if ((r = fvc_matrix_update_values_async(ctx, ad, au, au)) == FVC_OK)
      r = fvc_solve_async(ctx, code, b, s->xe, tol, s->o.maxit, &o, stp);
    fvc_context_set_stream(ctx, s->stream);
    return r;
  });
  if (rc != FVC_OK) return rc;
  fvc::set_ok<<<1, 1, 0, s->stream>>>(hok, s->gctr, s->rec, stp, sys);
  fvc::count_launch();
  return cap_if(s, hok, &s->launches_ok[sys], [&](cudaStream_t bs) {
    const int32_t r = fvc_getres(n, s->num, x_cells, s->xe, 0, bs);
    return r != FVC_OK ? r : after(bs);
  });
}

int32_t capture_iteration(fvc_simple *s, const cudaGraphConditionalHandle *h) {
  cudaStream_t st = s->stream;
  const int64_t l0 = fvc_kernel_launches();
  int64_t body = 0;
  auto none = [](cudaStream_t) { return (int32_t)FVC_OK; };
  auto dots = [&](int off, int k) {
    fvc::rec_dots<<<1, 1, 0, st>>>(s->gctr, s->rec, s->dots, off, k);
    fvc::count_launch();
  };
  auto run = [&](int sys, int dot, int use_sqrt) {
    fvc::set_run<<<1, 1, 0, st>>>(h[2 * sys], s->gctr, s->rec, dot, use_sqrt, sys);
    fvc::count_launch();
  };
  int32_t rc;
  if ((rc = stage_momentum(s, st)) != FVC_OK) {
    fprintf(stderr, "fvcgpu: graph capture: the momentum stage returned status %d\n", rc);
    return rc;
  }
  dots(0, 2);
  run(0, 0, 0);
  if ((rc = cap_solve(s, 0, s->ctx_u, s->o.code_u, s->ad1, s->au1, s->b1, s->u1, s->o.tol_u, h[0],
                      h[1], none)) != FVC_OK)
    return rc;
  run(1, 1, 0);
  if ((rc = cap_solve(s, 1, s->ctx_u, s->o.code_u, s->ad2, s->au2, s->b2, s->u2, s->o.tol_u, h[2],
                      h[3], none)) != FVC_OK)
    return rc;
  if ((rc = stage_pressure(s, st)) != FVC_OK) return rc;
  dots(2, 3);
  run(2, 4, 1);
  if ((rc = cap_solve(s, 2, s->ctx_pc, s->o.code_pc, s->adp, s->aup, s->bp, s->pc, s->o.tol_pc,
                      h[4], h[5], [&](cudaStream_t bs) { return after_pressure(s, bs); })) !=
      FVC_OK)
    return rc;
  if (s->gas) {
    if ((rc = stage_energy(s, st)) != FVC_OK) return rc;
    dots(5, 2);
    run(3, 5, 1);
    if ((rc = cap_solve(s, 3, s->ctx_e, 2, s->ade, s->aue, s->be, s->en, s->o.tol_u, h[6], h[7],
                        [&](cudaStream_t bs) { return after_energy(s, bs); })) != FVC_OK)
      return rc;
  }
  fvc::next_rec<<<1, 1, 0, st>>>(s->gctr);
  fvc::count_launch();
  for (int k = 0; k < 4; ++k) body += s->launches_run[k] + s->launches_ok[k];
  s->launches_top = fvc_kernel_launches() - l0 - body;
  return FVC_OK;
}

void drop_graph(fvc_simple *s) {
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  if (s->graph) cudaGraphDestroy(s->graph);
  s->gexec = nullptr;
  s->graph = nullptr;
}

int32_t build_graph(fvc_simple *s) {
  drop_graph(s);
  int32_t rc;
  if (!s->rec) {
    if ((rc = dalloc(s, s->rec, fvc::kRecMax)) != FVC_OK || (rc = dalloc(s, s->gctr, 2)) != FVC_OK ||
        (rc = dalloc(s, s->st_tmp, 16)) != FVC_OK)
      return rc;
    if (cudaMallocHost(&s->h_rec, sizeof(fvc::SimpleRec) * fvc::kRecMax) != cudaSuccess)
      return FVC_ERR_CUDA;
  }
  if (!s->body && cudaStreamCreateWithFlags(&s->body, cudaStreamNonBlocking) != cudaSuccess)
    return FVC_ERR_CUDA;
  // every solve's scratch exists before the capture
  fvc_context *ctxs[3] = {s->ctx_u, s->ctx_pc, s->ctx_e};
  const int codes[3] = {s->o.code_u, s->o.code_pc, 2};
  for (int k = 0; k < (s->gas ? 3 : 2); ++k)
    if ((rc = fvc::context_prepare(ctxs[k], codes[k], solve_opts(s, ctxs[k]))) != FVC_OK)
      return rc;
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return FVC_ERR_CUDA;
  const int64_t l0 = fvc_kernel_launches();
  if (!cap_ok(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeRelaxed),
              "cudaStreamBeginCapture"))
    return FVC_ERR_CUDA;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  rc = FVC_OK;
  // run/ok handles of u1, u2, p' (and the energy): every handle created
  // must belong to a conditional node, or the instantiation fails
  cudaGraphConditionalHandle h[8];
  if (!cap_ok(cudaStreamGetCaptureInfo(s->stream, &cs, nullptr, &g), "cudaStreamGetCaptureInfo"))
    rc = FVC_ERR_CUDA;
  for (int k = 0; k < (s->gas ? 8 : 6) && rc == FVC_OK; ++k)
    if (!cap_ok(cudaGraphConditionalHandleCreate(&h[k], g, 0, cudaGraphCondAssignDefault),
                "cudaGraphConditionalHandleCreate"))
      rc = FVC_ERR_CUDA;
  if (rc == FVC_OK) rc = capture_iteration(s, h);
  cudaGraph_t out = nullptr;
  const bool ended = cap_ok(cudaStreamEndCapture(s->stream, &out), "cudaStreamEndCapture");
  // launches were counted at the capture; they are counted per replay instead
  fvc::count_launch(l0 - fvc_kernel_launches());
  if (rc == FVC_OK && !ended) rc = FVC_ERR_CUDA;
  if (rc == FVC_OK) {
    cudaGraphInstantiateParams ip;
    memset(&ip, 0, sizeof(ip));
    if (!cap_ok(cudaGraphInstantiateWithParams(&s->gexec, out, &ip),
                "cudaGraphInstantiateWithParams")) {
      cudaGraphNodeType t = cudaGraphNodeTypeEmpty;
      if (ip.errNode_out) cudaGraphNodeGetType(ip.errNode_out, &t);
      fprintf(stderr, "fvcgpu: graph capture: instantiation result %d, node type %d\n",
              (int)ip.result_out, ip.errNode_out ? (int)t : -1);
      rc = FVC_ERR_CUDA;
    }
  }
  if (rc != FVC_OK) {
    if (out) cudaGraphDestroy(out);
    cudaGetLastError();
    fprintf(stderr, "fvcgpu: the SIMPLE iteration could not be captured as a CUDA graph "
                    "(status %d)\n", rc);
    return rc;
  }
  s->graph = out;
  s->graph_gas = s->gas;
  return FVC_OK;
}

const char *const kSysName[4] = {"u1", "u2", "p'", "energy"};

// nit outer iterations as graph launches, in batches of at most kRecMax with
// one synchronisation each; the same results as iterate_plain
int32_t iterate_graph(fvc_simple *s, int32_t nit, double *res, int32_t *its, int nrep) {
  int32_t rc;
  if (!s->gexec || s->graph_gas != s->gas)
    if ((rc = build_graph(s)) != FVC_OK) return rc;
  cudaStream_t st = s->stream;
  for (int done = 0; done < nit;) {
    const int chunk = std::min(fvc::kRecMax, nit - done);
    cudaMemsetAsync(s->rec, 0, sizeof(fvc::SimpleRec) * chunk, st);
    cudaMemsetAsync(s->gctr, 0, 2 * sizeof(int32_t), st);
    for (int c = 0; c < chunk; ++c)
      if (cudaGraphLaunch(s->gexec, st) != cudaSuccess) return FVC_ERR_CUDA;
    cudaMemcpyAsync(s->h_rec, s->rec, sizeof(fvc::SimpleRec) * chunk, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(s->h_err, s->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return FVC_ERR_CUDA;
    if (*s->h_err) return FVC_ERR_UNSUPPORTED;  // a velocity boundary code outside 0..4
    int64_t launched = s->launches_top * chunk;
    for (int c = 0; c < chunk; ++c) {
      const fvc::SimpleRec &r = s->h_rec[c];
      for (int k = 0; k < 4; ++k) {
        launched += (r.ran[k] ? s->launches_run[k] : 0) + (r.ok[k] ? s->launches_ok[k] : 0);
        if (r.ran[k] && !r.ok[k]) {
          fvc::count_launch(launched);
          const fvc_opts so = solve_opts(s, k == 2 ? s->ctx_pc : s->ctx_u);
          fprintf(stderr, "fvcgpu: SIMPLE %s solve (code %d, %s) ended with status %d after %d "
                          "iterations\n", kSysName[k],
                  k < 2 ? s->o.code_u : k == 2 ? s->o.code_pc : 2,
                  so.precision == FVC_PREC_MIXED ? "mixed" : "fp64", r.st[k][0], r.st[k][1]);
          return r.st[k][0];
        }
      }
      const int it = done + c;
      if (res) {
        res[nrep * it] = std::sqrt(r.dots[2]);
        res[nrep * it + 1] = std::sqrt(r.dots[3]);
        res[nrep * it + 2] = std::sqrt(r.dots[4]);
        if (nrep == 4)
          res[4 * it + 3] = r.ran[3] ? std::sqrt(r.dots[6]) : std::sqrt(r.dots[5]);
      }
      if (its)
        for (int k = 0; k < nrep; ++k) its[nrep * it + k] = r.ran[k] ? r.st[k][1] : 0;
    }
    fvc::count_launch(launched);
    done += chunk;
  }
  return FVC_OK;
}

int32_t iterate(fvc_simple *s, int32_t nit, double *res, int32_t *its, int nrep) {
  if (!s || nit < 0) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  return s->use_graph ? iterate_graph(s, nit, res, its, nrep)
                      : iterate_plain(s, nit, res, its, nrep);
}

}  // namespace

extern "C" {

int32_t fvc_simple_set_graph(fvc_simple *s, int32_t on) {
  if (!s) return FVC_ERR_ARG;
  s->use_graph = on != 0;
  if (!on) drop_graph(s);
  return FVC_OK;
}

int32_t fvc_simple_iterate(fvc_simple *s, int32_t nit, double *res, int32_t *its) {
  return iterate(s, nit, res, its, 3);
}

int32_t fvc_simple_iterate_energy(fvc_simple *s, int32_t nit, double *res, int32_t *its) {
  if (!s || !s->gas) return FVC_ERR_ARG;
  return iterate(s, nit, res, its, 4);
}

int32_t fvc_simple_energy(fvc_simple *s, const int32_t *pedge_e, const double *sedge_e,
                          double gx, double gy, double t0) {
  if (!s || !pedge_e || !sedge_e || s->gas || s->cp == 0.0) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  const size_t n = s->numel, ld = s->nshared + 1;
  int32_t rc;
  if ((rc = dcopy(s, s->pedge_e, pedge_e, ld * n)) != FVC_OK ||
      (rc = dcopy(s, s->sedge_e, sedge_e, ld * n)) != FVC_OK ||
      (rc = make_system(s, s->ident, 1, &s->ctx_e, &s->ia_e, &s->ja_e, &s->nja_e)) != FVC_OK)
    return rc;
  double **vec[] = {&s->en, &s->en0, &s->temp, &s->ade, &s->be, &s->be0, &s->rce};
  for (double **v : vec)
    if ((rc = dalloc(s, *v, n)) != FVC_OK) return rc;
  if ((rc = dalloc(s, s->ro, 3 * n)) != FVC_OK || (rc = dalloc(s, s->ge, 2 * n)) != FVC_OK ||
      (rc = dalloc(s, s->aue, s->nja_e)) != FVC_OK)
    return rc;
  s->grav[0] = gx;
  s->grav[1] = gy;
  // start-up of src/Main.f:815-837: T uniform, h from T, en0 = en, w0 = w,
  // the three density levels from the ideal-gas law
  fill<<<fvc::g((int)n), fvc::kT, 0, s->stream>>>((int)n, s->temp, t0);
  fvc::count_launch();
  if ((rc = fvc_cells_enthalpy_temperature((int)n, s->en, s->temp, s->cp, s->tref, 0,
                                           s->stream)) != FVC_OK)
    return rc;
  cudaMemcpyAsync(s->en0, s->en, sizeof(double) * n, cudaMemcpyDeviceToDevice, s->stream);
  cudaMemcpyAsync(s->w0, s->w, sizeof(double) * 2 * n, cudaMemcpyDeviceToDevice, s->stream);
  for (int row = 1; row <= 3; ++row)
    if ((rc = fvc_cells_ideal_gas_density((int)n, s->ro, s->temp, 1, row, 1.0, 1.0,
                                          s->stream)) != FVC_OK)
      return rc;
  s->gas = true;
  if ((rc = time_term_gas(s)) != FVC_OK) return rc;
  return cudaStreamSynchronize(s->stream) == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_simple_energy_fields(const fvc_simple *s, double *temp, double *en, double *ro) {
  if (!s || !s->gas) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  const size_t n = s->numel;
  if (temp && cudaMemcpyAsync(temp, s->temp, sizeof(double) * n, cudaMemcpyDeviceToHost,
                              s->stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  if (en && cudaMemcpyAsync(en, s->en, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream) !=
                cudaSuccess)
    return FVC_ERR_CUDA;
  if (ro && cudaMemcpyAsync(ro, s->ro, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost,
                            s->stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  return cudaStreamSynchronize(s->stream) == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_simple_fields(const fvc_simple *s, double *w, double *p) {
  if (!s) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  if (w && cudaMemcpyAsync(w, s->w, sizeof(double) * 2 * s->numel, cudaMemcpyDeviceToHost,
                           s->stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  if (p && cudaMemcpyAsync(p, s->p, sizeof(double) * s->numel, cudaMemcpyDeviceToHost,
                           s->stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  return cudaStreamSynchronize(s->stream) == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_simple_set_fields(fvc_simple *s, const double *w, const double *p) {
  if (!s) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  if (w && cudaMemcpyAsync(s->w, w, sizeof(double) * 2 * s->numel, cudaMemcpyHostToDevice,
                           s->stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  if (p && cudaMemcpyAsync(s->p, p, sizeof(double) * s->numel, cudaMemcpyHostToDevice,
                           s->stream) != cudaSuccess)
    return FVC_ERR_CUDA;
  return cudaStreamSynchronize(s->stream) == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_simple_system(const fvc_simple *s, int32_t which, double *ad, double *au, double *b,
                          int64_t *nja) {
  if (!s || which < 1 || which > 4 || (which == 4 && !s->gas)) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  const double *dad = which == 1 ? s->ad1 : which == 2 ? s->ad2 : which == 3 ? s->adp : s->ade;
  const double *dau = which == 1 ? s->au1 : which == 2 ? s->au2 : which == 3 ? s->aup : s->aue;
  const double *db = which == 1 ? s->b1 : which == 2 ? s->b2 : which == 3 ? s->bp : s->be;
  const size_t na = which <= 2 ? s->nja_u : which == 3 ? s->nja_pc : s->nja_e;
  const size_t n = (size_t)s->numel;
  if (nja) *nja = (int64_t)na;
  if (ad && cudaMemcpyAsync(ad, dad, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream) !=
                cudaSuccess)
    return FVC_ERR_CUDA;
  if (au && cudaMemcpyAsync(au, dau, sizeof(double) * na, cudaMemcpyDeviceToHost, s->stream) !=
                cudaSuccess)
    return FVC_ERR_CUDA;
  if (b && cudaMemcpyAsync(b, db, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream) !=
               cudaSuccess)
    return FVC_ERR_CUDA;
  return cudaStreamSynchronize(s->stream) == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_simple_get_state(const fvc_simple *s, double *w, double *w0, double *p, double *en,
                             double *en0, double *ro) {
  if (!s || (!s->gas && (en || en0 || ro))) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  const size_t n = s->numel;
  const struct {
    double *h;
    const double *d;
    size_t k;
  } cp[] = {{w, s->w, 2 * n}, {w0, s->w0, 2 * n}, {p, s->p, n},
            {en, s->en, n},   {en0, s->en0, n}, {ro, s->ro, 3 * n}};
  for (const auto &c : cp)
    if (c.h && cudaMemcpyAsync(c.h, c.d, sizeof(double) * c.k, cudaMemcpyDeviceToHost,
                               s->stream) != cudaSuccess)
      return FVC_ERR_CUDA;
  return cudaStreamSynchronize(s->stream) == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_simple_set_state(fvc_simple *s, const double *w, const double *w0, const double *p,
                             const double *en, const double *en0, const double *ro) {
  if (!s || (!s->gas && (en || en0 || ro))) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  const size_t n = s->numel;
  const struct {
    const double *h;
    double *d;
    size_t k;
  } cp[] = {{w, s->w, 2 * n}, {w0, s->w0, 2 * n}, {p, s->p, n},
            {en, s->en, n},   {en0, s->en0, n}, {ro, s->ro, 3 * n}};
  for (const auto &c : cp)
    if (c.h && cudaMemcpyAsync(c.d, c.h, sizeof(double) * c.k, cudaMemcpyHostToDevice,
                               s->stream) != cudaSuccess)
      return FVC_ERR_CUDA;
  // the start of a step from the loaded levels: time terms (and w0 = w,
  // en0 = en); with the energy equation the temperature from the enthalpy
  int32_t rc;
  if (s->gas) {
    if ((rc = fvc_cells_enthalpy_temperature((int)n, s->en, s->temp, s->cp, s->tref, 1,
                                             s->stream)) != FVC_OK ||
        (rc = time_term_gas(s)) != FVC_OK)
      return rc;
  } else {
    if ((rc = time_term(s)) != FVC_OK) return rc;
    if (cudaMemcpyAsync(s->w0, s->w, sizeof(double) * 2 * n, cudaMemcpyDeviceToDevice,
                        s->stream) != cudaSuccess)
      return FVC_ERR_CUDA;
  }
  return cudaStreamSynchronize(s->stream) == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_simple_destroy(fvc_simple *s) {
  if (!s) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  cudaStreamSynchronize(s->stream);
  release(s);
  delete s;
  return FVC_OK;
}

}  // extern "C"
