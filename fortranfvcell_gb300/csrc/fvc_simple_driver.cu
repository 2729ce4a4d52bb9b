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
#include <algorithm>
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
  void *geo = nullptr;  // the cells' geometry, computed once (m.geometry)
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
  if (s->geo) fvc_cells_geometry_destroy(s->geo);
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
  // the cell geometry once (the cell kernels would otherwise recompute it,
  // in FP64, in every kernel of every outer iteration), once the mesh
  // arrays have landed
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return fail(FVC_ERR_CUDA);
  if ((rc = fvc_cells_geometry_create(&s->m, &s->geo)) != FVC_OK) return fail(rc);
  s->m.geometry = s->geo;
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

// ---- many cases advanced together (fvc_simple_batch) -----------------------
// The outer iterations of ncases independent SIMPLE loops (each an
// fvc_simple, created by the caller), with every linear solve of a stage
// in one persistent launch: all u1 and u2 systems together, then all p'
// systems, then all enthalpy systems.  Each stage's systems are the
// diagonal blocks of one matrix on one solver context (each system padded
// with identity rows to a multiple of 32 rows); a pack kernel gathers the
// cases' freshly assembled values, right-hand sides and unknowns into it,
// the batched launch solves every system with its own convergence test and
// status, an unpack kernel scatters the unknowns back.  The reference's
// test before each solve (Simple.f: no solve when the right-hand side's or
// the residual's norm is below 1e-32) becomes a per-system mask read by the
// launch, and the work after a p' or enthalpy solve (its gradient and
// simpleUpdate, the temperatures and densities) runs inside a conditional
// graph node per case.  One outer iteration of all cases is one CUDA graph.

namespace fvc {
namespace {

// One system of a stage: where its values and unknown live in its case,
// where they go in the stage's block-diagonal arrays, and the reference's
// test before its solve.
struct StageSeg {
  const double *ad, *au, *b;  // the case's system, equation order (au: nad values)
  double *x;                  // the case's unknown, cell order
  const int32_t *num;         // cell -> equation (1-based)
  const double *dots;         // the case's norms of this stage
  int n, nad, row0;           // rows, off-diagonals, first row in the stage matrix
  int dot, use_sqrt;          // solve when dots[dot] (or its square root) >= 1e-32
  long long au0;              // first off-diagonal in the stage matrix
};

// values, right-hand sides and unknowns (to equation order) into the stage
// arrays; the mask from the reference's test.  blockIdx.y = system.
__global__ void stage_pack(const StageSeg *segs, double *ad, double *au, double *b, double *x,
                           int32_t *run) {
  const StageSeg g = segs[blockIdx.y];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < g.n) {
    ad[g.row0 + i] = g.ad[i];
    b[g.row0 + i] = g.b[i];
    x[g.row0 + g.num[i] - 1] = g.x[i];
  }
  if (i < g.nad) au[g.au0 + i] = g.au[i];
  if (i == 0) {
    const double v = g.use_sqrt ? sqrt(g.dots[g.dot]) : g.dots[g.dot];
    run[blockIdx.y] = (v >= 1.0e-32) ? 1 : 0;
  }
}

// the unknowns back to the cases (a masked system gives back what it got)
__global__ void stage_unpack(const StageSeg *segs, const double *x) {
  const StageSeg g = segs[blockIdx.y];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < g.n) g.x[i] = x[g.row0 + g.num[i] - 1];
}

// per case: run the work after its solve when the solve ran and ended with
// FVC_OK (the batched launch's status slots: 16 ints per system, [1] status)
struct CondSet {
  const cudaGraphConditionalHandle *h;
  const int32_t *run;
  const int32_t *status;  // per system, after an FP64 finish where one ran
  int ncases;
};
__global__ void stage_conds(CondSet a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.ncases) return;
  const unsigned int go = (a.run[c] != 0 && a.status[c] == FVC_OK) ? 1u : 0u;
  cudaGraphSetConditional(a.h[c], go);
}

// each case's norms (k of them, from its dots) into its record slots
__global__ void rec_case_dots(const double *const *dots, int ncases, int k, int off,
                              double *rec) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncases) return;
  for (int i = 0; i < k; ++i) rec[5 * (size_t)c + off + i] = dots[c][i];
}

// a mixed stage's systems to finish in FP64: BiCGSTAB systems that ran and
// whose FP32 sweeps stalled (FVC_ERR_NOCONV before max_refine sweeps and
// maxit iterations: the kernel's stall rule), as a synchronous mixed solve
// finishes them
__global__ void stall_mask(const int32_t *run, const int32_t *codes, const int *ires, int nsys,
                           int max_refine, int maxit, int32_t *run2) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const int *r = ires + 16 * s;
  run2[s] = (run[s] && codes[s] == 2 && r[1] == FVC_ERR_NOCONV && r[0] < max_refine &&
             r[2] < maxit)
                ? 1
                : 0;
}

// each system of a stage: its status (after an FP64 finish where one ran)
// for the conditional nodes, and its record: run, status, iterations (FP32
// plus FP64 for mixed), FP32 iterations
__global__ void stage_result(const int32_t *run, const int *ires, const int32_t *run2,
                             const int *ires64, int nsys, int mixed, int32_t *status,
                             int32_t *rec) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const bool fin = run2 && run2[s];
  const int st = !run[s] ? FVC_OK : (fin ? ires64[16 * s + 1] : ires[16 * s + 1]);
  const int inner = run[s] ? (mixed ? ires[16 * s + 2] : 0) : 0;
  const int its = !run[s] ? 0 : (mixed ? inner + (fin ? ires64[16 * s] : 0) : ires[16 * s]);
  status[s] = st;
  rec[4 * (size_t)s] = run[s];
  rec[4 * (size_t)s + 1] = st;
  rec[4 * (size_t)s + 2] = its;
  rec[4 * (size_t)s + 3] = inner;
}

// the cases' gradient error words, or-ed
__global__ void rec_errs(const int32_t *const *errs, int ncases, int32_t *out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncases && *errs[c] != 0) atomicOr(out, 1);
}

}  // namespace
}  // namespace fvc

struct fvc_simple_batch {
  int device = 0, ncases = 0;
  cudaStream_t stream = nullptr, body = nullptr;
  // the cases' cell kernels and conditional nodes run on kBranches
  // streams side by side (case c on branch c mod kBranches), forked from
  // and joined back into stream: each case's kernels are small, so one
  // stream would leave most of the device idle between them
  static constexpr int kBranches = 16;
  cudaStream_t branch[kBranches] = {};
  cudaEvent_t fork = nullptr, join[kBranches] = {};
  bool gas = false;
  int precision = FVC_PREC_FP64;    // p'
  int precision_u = FVC_PREC_FP64;  // u, v and the enthalpy
  std::vector<fvc_simple *> cs;
  struct Stage {
    int nsys = 0, maxlen = 0;
    fvc_context *ctx = nullptr;
    std::vector<int32_t> row_start, codes, inits, sys_case, sys_which;
    std::vector<double> tols, hints;
    fvc::StageSeg *segs = nullptr;  // device
    double *ad = nullptr, *au = nullptr, *b = nullptr, *x = nullptr;
    int32_t *run = nullptr;
    fvc::BatchPlan plan;
    int32_t *rec = nullptr;     // device: 4 per system
    int32_t *status = nullptr;  // device: per system, the final status
    // mixed stages with BiCGSTAB systems: the FP64 finish of stalled ones
    bool finish = false;
    fvc::BatchPlan plan64;
    int32_t *run2 = nullptr, *codes_d = nullptr;
  } st[3];                   // 0 u1+u2, 1 p', 2 enthalpy
  double **d_dots = nullptr;    // device array of the cases' dots pointers
  int32_t **d_errs = nullptr;   // and of their gradient error words
  double *rec_dots = nullptr;   // device: 5 per case
  int32_t *rec_err = nullptr;
  double *h_dots = nullptr;     // pinned copies
  int32_t *h_sys = nullptr, *h_err = nullptr;
  cudaGraphConditionalHandle *h_handles = nullptr;  // pinned
  cudaGraphConditionalHandle *d_handles = nullptr;  // device: p' then enthalpy, per case
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int64_t launches_top = 0;
  std::vector<int64_t> launches_body[2];  // per case: after p', after the enthalpy
  int iterations_done = 0;
  bool hinted = false;
  std::vector<void *> owned;
};

namespace {

template <typename T>
int32_t balloc(fvc_simple_batch *B, T *&p, size_t n) {
  if (cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) return FVC_ERR_CUDA;
  B->owned.push_back(p);
  return cudaMemset(p, 0, sizeof(T) * std::max<size_t>(n, 1)) == cudaSuccess ? FVC_OK
                                                                             : FVC_ERR_CUDA;
}

void batch_drop_graph(fvc_simple_batch *B) {
  if (B->gexec) cudaGraphExecDestroy(B->gexec);
  if (B->graph) cudaGraphDestroy(B->graph);
  B->gexec = nullptr;
  B->graph = nullptr;
}

void batch_release(fvc_simple_batch *B) {
  batch_drop_graph(B);
  for (auto &S : B->st) {
    if (S.ctx) {
      fvc::context_free_batched(S.ctx, S.plan);
      fvc::context_free_batched(S.ctx, S.plan64);
      fvc_context_destroy(S.ctx);
    }
  }
  for (void *p : B->owned) cudaFree(p);
  if (B->h_dots) cudaFreeHost(B->h_dots);
  if (B->h_sys) cudaFreeHost(B->h_sys);
  if (B->h_err) cudaFreeHost(B->h_err);
  if (B->h_handles) cudaFreeHost(B->h_handles);
  if (B->body) cudaStreamDestroy(B->body);
  for (int k = 0; k < fvc_simple_batch::kBranches; ++k) {
    if (B->branch[k]) cudaStreamDestroy(B->branch[k]);
    if (B->join[k]) cudaEventDestroy(B->join[k]);
  }
  if (B->fork) cudaEventDestroy(B->fork);
  if (B->stream) cudaStreamDestroy(B->stream);
}

// A stage's block-diagonal structure on its context and its device arrays.
// which: 1 u1, 2 u2 (stage 0), 3 p' (stage 1), 4 enthalpy (stage 2).
int32_t batch_stage(fvc_simple_batch *B, int k, const std::vector<std::vector<int32_t>> &ia_c,
                    const std::vector<std::vector<int32_t>> &ja_c) {
  fvc_simple_batch::Stage &S = B->st[k];
  const int per = (k == 0) ? 2 : 1;
  S.nsys = B->ncases * per;
  S.row_start.assign(S.nsys + 1, 0);
  std::vector<fvc::StageSeg> h((size_t)S.nsys);
  std::vector<int32_t> ia(1, 1), ja;
  long long au0 = 0;
  for (int c = 0; c < B->ncases; ++c) {
    fvc_simple *s = B->cs[c];
    const int n = s->numel;
    const int nad = ia_c[c][n] - 1;
    for (int q = 0; q < per; ++q) {
      const int sys = per * c + q, which = (k == 0) ? 1 + q : (k == 1 ? 3 : 4);
      const int row0 = S.row_start[sys];
      const int rows = (n + 31) / 32 * 32;
      S.row_start[sys + 1] = row0 + rows;
      fvc::StageSeg &g = h[sys];
      g.n = n;
      g.nad = nad;
      g.row0 = row0;
      g.au0 = au0;
      g.num = s->num;
      g.dots = s->dots;
      if (which == 1) {
        g.ad = s->ad1; g.au = s->au1; g.b = s->b1; g.x = s->u1; g.dot = 0; g.use_sqrt = 0;
      } else if (which == 2) {
        g.ad = s->ad2; g.au = s->au2; g.b = s->b2; g.x = s->u2; g.dot = 1; g.use_sqrt = 0;
      } else if (which == 3) {
        g.ad = s->adp; g.au = s->aup; g.b = s->bp; g.x = s->pc; g.dot = 2; g.use_sqrt = 1;
      } else {
        g.ad = s->ade; g.au = s->aue; g.b = s->be; g.x = s->en; g.dot = 0; g.use_sqrt = 1;
      }
      S.maxlen = std::max(S.maxlen, std::max(n, nad));
      // the case's rows (columns shifted), then identity rows to the slice
      for (int i = 0; i < n; ++i) {
        for (int q2 = ia_c[c][i] - 1; q2 < ia_c[c][i + 1] - 1; ++q2)
          ja.push_back(ja_c[c][q2] + row0);
        ia.push_back((int32_t)ja.size() + 1);
      }
      for (int i = n; i < rows; ++i) ia.push_back((int32_t)ja.size() + 1);
      au0 += nad;
      const int code = (which <= 2) ? s->o.code_u : (which == 3 ? s->o.code_pc : 2);
      S.codes.push_back(code);
      S.inits.push_back(fvc::context_default_init(code, 1));
      S.tols.push_back(which == 3 ? s->o.tol_pc : s->o.tol_u);
      S.sys_case.push_back(c);
      S.sys_which.push_back(which);
    }
  }
  const int N = S.row_start[S.nsys];
  const long long NAD = au0;
  if (NAD > INT32_MAX - 1) return FVC_ERR_ARG;
  int32_t rc;
  if ((rc = balloc(B, S.segs, (size_t)S.nsys)) != FVC_OK || (rc = balloc(B, S.ad, N)) != FVC_OK ||
      (rc = balloc(B, S.au, (size_t)NAD)) != FVC_OK || (rc = balloc(B, S.b, N)) != FVC_OK ||
      (rc = balloc(B, S.x, N)) != FVC_OK || (rc = balloc(B, S.run, (size_t)S.nsys)) != FVC_OK ||
      (rc = balloc(B, S.rec, 4 * (size_t)S.nsys)) != FVC_OK ||
      (rc = balloc(B, S.status, (size_t)S.nsys)) != FVC_OK ||
      (rc = balloc(B, S.run2, (size_t)S.nsys)) != FVC_OK ||
      (rc = balloc(B, S.codes_d, (size_t)S.nsys)) != FVC_OK)
    return rc;
  if (cudaMemcpy(S.codes_d, S.codes.data(), sizeof(int32_t) * S.nsys, cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return FVC_ERR_CUDA;
  if (cudaMemcpy(S.segs, h.data(), sizeof(fvc::StageSeg) * S.nsys, cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return FVC_ERR_CUDA;
  // identity on the padding rows (the systems' own rows are packed later)
  std::vector<double> ones((size_t)N, 1.0), zeros((size_t)std::max<long long>(NAD, 1), 0.0);
  if (cudaMemcpy(S.ad, ones.data(), sizeof(double) * N, cudaMemcpyHostToDevice) != cudaSuccess)
    return FVC_ERR_CUDA;
  if ((rc = fvc_context_create(&S.ctx, B->device)) != FVC_OK) return rc;
  fvc_context_set_stream(S.ctx, B->stream);
  return fvc_matrix_set(S.ctx, 1, 1, N, (int32_t)NAD, ones.data(), zeros.data(), zeros.data(),
                        ia.data(), ja.data());
}

// stage k's solver options: p' (stage 1) takes precision, u/v and the
// enthalpy precision_u
fvc_opts batch_opts(const fvc_simple_batch *B, int k) {
  fvc_opts o;
  fvc_opts_default(&o);
  o.precision = (k == 1) ? B->precision : B->precision_u;
  o.init = 1;
  return o;
}

// Plans every stage's launch (hints: the iterations each system took in the
// last outer iteration, else sqrt(rows)) and captures one outer iteration.
int32_t batch_build(fvc_simple_batch *B) {
  batch_drop_graph(B);
  const int nst = B->gas ? 3 : 2;
  int32_t rc;
  for (int k = 0; k < nst; ++k) {
    fvc_simple_batch::Stage &S = B->st[k];
    fvc::context_free_batched(S.ctx, S.plan);
    // the value path's buffers exist before the capture
    if ((rc = fvc_matrix_update_values_async(S.ctx, S.ad, S.au, S.au)) != FVC_OK) return rc;
    if ((rc = fvc::context_plan_batched(S.ctx, S.nsys, S.row_start.data(), S.codes.data(),
                                        S.tols.data(), S.hints.empty() ? nullptr : S.hints.data(),
                                        S.inits.data(), S.run, 0.0, batch_opts(B, k),
                                        S.plan)) != FVC_OK)
      return rc;
    // a mixed stage with BiCGSTAB systems: the FP64 plan that finishes the
    // stalled ones from their FP32 iterate (warm start), on ||r|| <= tol ||b||
    fvc::context_free_batched(S.ctx, S.plan64);
    S.finish = batch_opts(B, k).precision == FVC_PREC_MIXED &&
               std::find(S.codes.begin(), S.codes.end(), 2) != S.codes.end();
    if (S.finish) {
      fvc_opts f = batch_opts(B, k);
      f.precision = FVC_PREC_FP64;
      f.stop_rule = 1;
      const std::vector<int32_t> warm((size_t)S.nsys, 0);
      if ((rc = fvc::context_plan_batched(S.ctx, S.nsys, S.row_start.data(), S.codes.data(),
                                          S.tols.data(), nullptr, warm.data(), S.run2, 0.0, f,
                                          S.plan64)) != FVC_OK)
        return rc;
    }
  }
  if (cudaStreamSynchronize(B->stream) != cudaSuccess) return FVC_ERR_CUDA;
  cudaStream_t st = B->stream;
  const int64_t l0 = fvc_kernel_launches();
  if (!cap_ok(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture"))
    return FVC_ERR_CUDA;
  rc = FVC_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  const int nc = B->ncases;
  const int ncond = (B->gas ? 2 : 1) * nc;
  if (!cap_ok(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g), "cudaStreamGetCaptureInfo"))
    rc = FVC_ERR_CUDA;
  for (int k = 0; k < ncond && rc == FVC_OK; ++k)
    if (!cap_ok(cudaGraphConditionalHandleCreate(&B->h_handles[k], g, 0,
                                                 cudaGraphCondAssignDefault),
                "cudaGraphConditionalHandleCreate"))
      rc = FVC_ERR_CUDA;
  if (rc == FVC_OK &&
      !cap_ok(cudaMemcpyAsync(B->d_handles, B->h_handles,
                              sizeof(cudaGraphConditionalHandle) * ncond, cudaMemcpyHostToDevice,
                              st),
              "cudaMemcpyAsync (handles)"))
    rc = FVC_ERR_CUDA;
  auto solve_stage = [&](int k) -> int32_t {
    fvc_simple_batch::Stage &S = B->st[k];
    const unsigned gx = (unsigned)((S.maxlen + fvc::kT - 1) / fvc::kT);
    fvc::stage_pack<<<dim3(gx, (unsigned)S.nsys), fvc::kT, 0, st>>>(S.segs, S.ad, S.au, S.b, S.x,
                                                                    S.run);
    fvc::count_launch();
    int32_t r = fvc_matrix_update_values_async(S.ctx, S.ad, S.au, S.au);
    if (r != FVC_OK) return r;
    const fvc_opts o = batch_opts(B, k);
    const int maxit = B->cs[0]->o.maxit;
    if ((r = fvc::context_enqueue_batched(S.ctx, S.plan, S.b, S.x, maxit, o)) != FVC_OK) return r;
    if (S.finish) {
      fvc::stall_mask<<<(S.nsys + 127) / 128, 128, 0, st>>>(S.run, S.codes_d, S.plan.ires,
                                                            S.nsys, 30, maxit, S.run2);
      fvc::count_launch();
      fvc_opts f = o;
      f.precision = FVC_PREC_FP64;
      f.stop_rule = 1;
      if ((r = fvc::context_enqueue_batched(S.ctx, S.plan64, S.b, S.x, maxit, f)) != FVC_OK)
        return r;
    }
    fvc::stage_result<<<(S.nsys + 127) / 128, 128, 0, st>>>(
        S.run, S.plan.ires, S.finish ? S.run2 : nullptr, S.finish ? S.plan64.ires : nullptr,
        S.nsys, o.precision == FVC_PREC_MIXED ? 1 : 0, S.status, S.rec);
    fvc::count_launch();
    fvc::stage_unpack<<<dim3(gx, (unsigned)S.nsys), fvc::kT, 0, st>>>(S.segs, S.x);
    fvc::count_launch();
    return FVC_OK;
  };
  // every case's part of a stage, case c on branch c mod kBranches: fork
  // the branches from st, enqueue, join them back (event waits; in the
  // capture these are the graph's parallel branches)
  constexpr int kB = fvc_simple_batch::kBranches;
  auto per_case = [&](auto &&f) -> int32_t {
    if (!cap_ok(cudaEventRecord(B->fork, st), "cudaEventRecord (fork)")) return FVC_ERR_CUDA;
    for (int k = 0; k < kB; ++k)
      if (!cap_ok(cudaStreamWaitEvent(B->branch[k], B->fork, 0), "cudaStreamWaitEvent (fork)"))
        return FVC_ERR_CUDA;
    int32_t r = FVC_OK;
    for (int c = 0; c < nc && r == FVC_OK; ++c) r = f(c, B->branch[c % kB]);
    for (int k = 0; k < kB; ++k)
      if (!cap_ok(cudaEventRecord(B->join[k], B->branch[k]), "cudaEventRecord (join)") ||
          !cap_ok(cudaStreamWaitEvent(st, B->join[k], 0), "cudaStreamWaitEvent (join)"))
        r = FVC_ERR_CUDA;
    return r;
  };
  // IF(the case's solve ran and ended FVC_OK) { after(case) } for every case
  auto after_stage = [&](int k, int hoff, int which) -> int32_t {
    fvc_simple_batch::Stage &S = B->st[k];
    fvc::CondSet a{B->d_handles + hoff, S.run, S.status, nc};
    fvc::stage_conds<<<(nc + 127) / 128, 128, 0, st>>>(a);
    fvc::count_launch();
    return per_case([&](int c, cudaStream_t bst) -> int32_t {
      fvc_simple *s = B->cs[c];
      // cap_if adds the node on the case's stream and captures the body
      // into the case's body stream: point them at the branch and ours
      cudaStream_t keep_stream = s->stream, keep_body = s->body;
      s->stream = bst;
      s->body = B->body;
      int64_t nl = 0;
      const int32_t r = cap_if(s, B->h_handles[hoff + c], &nl, [&](cudaStream_t bs) {
        return which == 3 ? after_pressure(s, bs) : after_energy(s, bs);
      });
      s->stream = keep_stream;
      s->body = keep_body;
      B->launches_body[which == 3 ? 0 : 1][c] = nl;
      return r;
    });
  };
  if (rc == FVC_OK)
    rc = per_case([&](int c, cudaStream_t bst) { return stage_momentum(B->cs[c], bst); });
  if (rc == FVC_OK) rc = solve_stage(0);
  if (rc == FVC_OK)
    rc = per_case([&](int c, cudaStream_t bst) { return stage_pressure(B->cs[c], bst); });
  if (rc == FVC_OK) {
    fvc::rec_case_dots<<<(nc + 127) / 128, 128, 0, st>>>(B->d_dots, nc, 3, 0, B->rec_dots);
    fvc::count_launch();
    rc = solve_stage(1);
  }
  if (rc == FVC_OK) rc = after_stage(1, 0, 3);
  if (B->gas) {
    if (rc == FVC_OK)
      rc = per_case([&](int c, cudaStream_t bst) { return stage_energy(B->cs[c], bst); });
    if (rc == FVC_OK) {
      fvc::rec_case_dots<<<(nc + 127) / 128, 128, 0, st>>>(B->d_dots, nc, 2, 3, B->rec_dots);
      fvc::count_launch();
      rc = solve_stage(2);
    }
    if (rc == FVC_OK) rc = after_stage(2, nc, 4);
  }
  if (rc == FVC_OK) {
    cudaMemsetAsync(B->rec_err, 0, sizeof(int32_t), st);
    fvc::rec_errs<<<(nc + 127) / 128, 128, 0, st>>>(B->d_errs, nc, B->rec_err);
    fvc::count_launch();
  }
  cudaGraph_t out = nullptr;
  const bool ended = cap_ok(cudaStreamEndCapture(st, &out), "cudaStreamEndCapture");
  int64_t body = 0;
  for (int q = 0; q < 2; ++q)
    for (int64_t v : B->launches_body[q]) body += v;
  B->launches_top = fvc_kernel_launches() - l0 - body;
  fvc::count_launch(l0 - fvc_kernel_launches());  // counted per replay instead
  if (rc == FVC_OK && !ended) rc = FVC_ERR_CUDA;
  if (rc == FVC_OK) {
    cudaGraphInstantiateParams ip;
    memset(&ip, 0, sizeof(ip));
    if (!cap_ok(cudaGraphInstantiateWithParams(&B->gexec, out, &ip),
                "cudaGraphInstantiateWithParams"))
      rc = FVC_ERR_CUDA;
  }
  if (rc != FVC_OK) {
    if (out) cudaGraphDestroy(out);
    cudaGetLastError();
    fprintf(stderr, "fvcgpu: the batched SIMPLE iteration could not be captured (status %d)\n",
            rc);
    return rc;
  }
  B->graph = out;
  return FVC_OK;
}

const char *const kBatchSys[4] = {"u1", "u2", "p'", "energy"};

// one outer iteration of every case: the graph launch, then its record
int32_t batch_step(fvc_simple_batch *B, int it, double *res, int32_t *its) {
  cudaStream_t st = B->stream;
  const int nc = B->ncases, nrep = B->gas ? 4 : 3, nst = B->gas ? 3 : 2;
  if (cudaGraphLaunch(B->gexec, st) != cudaSuccess) return FVC_ERR_CUDA;
  cudaMemcpyAsync(B->h_dots, B->rec_dots, sizeof(double) * 5 * nc, cudaMemcpyDeviceToHost, st);
  size_t off = 0;
  for (int k = 0; k < nst; ++k) {
    cudaMemcpyAsync(B->h_sys + off, B->st[k].rec, sizeof(int32_t) * 4 * B->st[k].nsys,
                    cudaMemcpyDeviceToHost, st);
    off += 4 * (size_t)B->st[k].nsys;
  }
  cudaMemcpyAsync(B->h_err, B->rec_err, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return FVC_ERR_CUDA;
  if (*B->h_err) return FVC_ERR_UNSUPPORTED;  // a velocity boundary code outside 0..4
  int64_t launched = B->launches_top;
  int32_t status = FVC_OK;
  off = 0;
  for (int k = 0; k < nst; ++k) {
    fvc_simple_batch::Stage &S = B->st[k];
    for (int sy = 0; sy < S.nsys; ++sy) {
      const int32_t *r = B->h_sys + off + 4 * (size_t)sy;
      const int c = S.sys_case[sy], which = S.sys_which[sy];
      if (its) its[((size_t)it * nc + c) * nrep + (which - 1)] = r[0] ? r[2] : 0;
      if (r[0] && r[1] == FVC_OK && which >= 3) launched += B->launches_body[which - 3][c];
      if (r[0] && r[1] != FVC_OK && status == FVC_OK) {
        fprintf(stderr, "fvcgpu: SIMPLE batch: case %d, %s solve ended with status %d after %d "
                        "iterations\n", c, kBatchSys[which - 1], r[1], r[2]);
        status = r[1];
      }
      // the next plan's share of blocks follows the iterations it took
      if (r[0] && r[2] > 0) S.hints[sy] = (double)r[2];
    }
    off += 4 * (size_t)S.nsys;
  }
  fvc::count_launch(launched);
  if (res)
    for (int c = 0; c < nc; ++c) {
      const double *d = B->h_dots + 5 * (size_t)c;
      double *rr = res + ((size_t)it * nc + c) * nrep;
      rr[0] = std::sqrt(d[0]);
      rr[1] = std::sqrt(d[1]);
      rr[2] = std::sqrt(d[2]);
      if (nrep == 4) rr[3] = (std::sqrt(d[3]) >= 1.0e-32) ? std::sqrt(d[4]) : std::sqrt(d[3]);
    }
  return status;
}

}  // namespace

extern "C" {

int32_t fvc_simple_batch_create(fvc_simple_batch **out, int32_t ncases,
                                fvc_simple *const *cases, int32_t precision,
                                int32_t precision_u) {
  if (!out || ncases < 1 || !cases) return FVC_ERR_ARG;
  if (precision_u < 0) precision_u = precision;
  if ((precision != FVC_PREC_FP64 && precision != FVC_PREC_MIXED) ||
      (precision_u != FVC_PREC_FP64 && precision_u != FVC_PREC_MIXED))
    return FVC_ERR_UNSUPPORTED;
  *out = nullptr;
  fvc_simple *c0 = cases[0];
  if (!c0) return FVC_ERR_ARG;
  for (int c = 0; c < ncases; ++c) {
    const fvc_simple *s = cases[c];
    if (!s || s->device != c0->device || s->gas != c0->gas || s->o.matriz_u != 1 ||
        s->o.matriz_pc != 1 || s->o.maxit != c0->o.maxit)
      return FVC_ERR_ARG;
  }
  auto *B = new (std::nothrow) fvc_simple_batch();
  if (!B) return FVC_ERR_CUDA;
  B->device = c0->device;
  B->ncases = ncases;
  B->gas = c0->gas;
  B->precision = precision;
  B->precision_u = precision_u;
  B->cs.assign(cases, cases + ncases);
  cudaSetDevice(B->device);
  int32_t rc = FVC_OK;
  if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&B->body, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming) != cudaSuccess)
    rc = FVC_ERR_CUDA;
  for (int k = 0; k < fvc_simple_batch::kBranches && rc == FVC_OK; ++k)
    if (cudaStreamCreateWithFlags(&B->branch[k], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&B->join[k], cudaEventDisableTiming) != cudaSuccess)
      rc = FVC_ERR_CUDA;
  // every case's CSRD structure on the host (the one all its systems share)
  std::vector<std::vector<int32_t>> ia_c(ncases), ja_c(ncases);
  for (int c = 0; c < ncases && rc == FVC_OK; ++c) {
    fvc_simple *s = cases[c];
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) rc = FVC_ERR_CUDA;
    ia_c[c].resize(s->numel + 1);
    int32_t nad = 0;
    int64_t len = 0;
    if (rc == FVC_OK)
      rc = fvc_mesh_datastruc(s->ident.data(), s->numel, s->nshared, 1, 1, ia_c[c].data(),
                              nullptr, &nad, &len);
    ja_c[c].resize((size_t)std::max<int64_t>(len, 1));
    if (rc == FVC_OK)
      rc = fvc_mesh_datastruc(s->ident.data(), s->numel, s->nshared, 1, 1, ia_c[c].data(),
                              ja_c[c].data(), &nad, &len);
  }
  const int nst = B->gas ? 3 : 2;
  for (int k = 0; k < nst && rc == FVC_OK; ++k) rc = batch_stage(B, k, ia_c, ja_c);
  const int ncond = (B->gas ? 2 : 1) * ncases;
  size_t nsys_all = 0;
  for (int k = 0; k < nst; ++k) nsys_all += (size_t)B->st[k].nsys;
  if (rc == FVC_OK) {
    std::vector<double *> dots(ncases);
    std::vector<int32_t *> errs(ncases);
    for (int c = 0; c < ncases; ++c) {
      dots[c] = cases[c]->dots;
      errs[c] = cases[c]->d_err;
    }
    if ((rc = balloc(B, B->d_dots, ncases)) == FVC_OK && (rc = balloc(B, B->d_errs, ncases)) ==
        FVC_OK && (rc = balloc(B, B->rec_dots, 5 * (size_t)ncases)) == FVC_OK &&
        (rc = balloc(B, B->rec_err, 1)) == FVC_OK && (rc = balloc(B, B->d_handles, ncond)) == FVC_OK) {
      if (cudaMemcpy(B->d_dots, dots.data(), sizeof(double *) * ncases, cudaMemcpyHostToDevice) !=
              cudaSuccess ||
          cudaMemcpy(B->d_errs, errs.data(), sizeof(int32_t *) * ncases,
                     cudaMemcpyHostToDevice) != cudaSuccess)
        rc = FVC_ERR_CUDA;
    }
  }
  if (rc == FVC_OK &&
      (cudaMallocHost(&B->h_dots, sizeof(double) * 5 * ncases) != cudaSuccess ||
       cudaMallocHost(&B->h_sys, sizeof(int32_t) * 4 * nsys_all) != cudaSuccess ||
       cudaMallocHost(&B->h_err, sizeof(int32_t)) != cudaSuccess ||
       cudaMallocHost(&B->h_handles, sizeof(cudaGraphConditionalHandle) * ncond) != cudaSuccess))
    rc = FVC_ERR_CUDA;
  if (rc == FVC_OK) {
    for (int q = 0; q < 2; ++q) B->launches_body[q].assign(ncases, 0);
    for (int k = 0; k < nst; ++k) {
      B->st[k].hints.resize(B->st[k].nsys);
      for (int sy = 0; sy < B->st[k].nsys; ++sy)  // until measured: sqrt(rows)
        B->st[k].hints[sy] =
            std::sqrt((double)(B->st[k].row_start[sy + 1] - B->st[k].row_start[sy]));
    }
  }
  if (rc != FVC_OK) {
    batch_release(B);
    delete B;
    return rc;
  }
  *out = B;
  return FVC_OK;
}

int32_t fvc_simple_batch_iterate(fvc_simple_batch *B, int32_t nit, double *res, int32_t *its) {
  if (!B || nit < 0) return FVC_ERR_ARG;
  cudaSetDevice(B->device);
  for (int it = 0; it < nit; ++it) {
    // the first outer iteration runs on sqrt(rows) shares; the graph is
    // captured again once, with the iterations it took as the shares
    if (!B->gexec || (B->iterations_done >= 1 && !B->hinted)) {
      if (B->iterations_done >= 1) B->hinted = true;
      const int32_t rc = batch_build(B);
      if (rc != FVC_OK) return rc;
    }
    const int32_t rc = batch_step(B, it, res, its);
    ++B->iterations_done;
    if (rc != FVC_OK) return rc;
  }
  return FVC_OK;
}

int32_t fvc_simple_batch_destroy(fvc_simple_batch *B) {
  if (!B) return FVC_ERR_ARG;
  cudaSetDevice(B->device);
  cudaStreamSynchronize(B->stream);
  batch_release(B);
  delete B;
  return FVC_OK;
}

}  // extern "C"
