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
  for (void *ptr : s->owned) cudaFree(ptr);
  if (s->h_dots) cudaFreeHost(s->h_dots);
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

// x (cells) -> equation order, solve, back to cells
int32_t solve(fvc_simple *s, fvc_context *ctx, int code, const double *ad, const double *au,
              const double *b, double *x_cells, double tol, int *its, const char *what) {
  const int n = s->numel;
  int32_t rc = fvc_getres(n, s->num, x_cells, s->xe, 1, s->stream);
  if (rc != FVC_OK) return rc;
  if ((rc = fvc_matrix_update_values(ctx, ad, au, au)) != FVC_OK) return rc;
  fvc_opts o;
  fvc_opts_default(&o);
  // p' (ctx_pc) takes precision; momentum and energy precision_u when set
  o.precision = (ctx != s->ctx_pc && s->o.precision_u >= 0) ? s->o.precision_u : s->o.precision;
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
  if (cudaMallocHost(&s->h_dots, 4 * sizeof(double)) != cudaSuccess) return fail(FVC_ERR_CUDA);
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

int32_t iterate(fvc_simple *s, int32_t nit, double *res, int32_t *its, int nrep) {
  if (!s || nit < 0) return FVC_ERR_ARG;
  cudaSetDevice(s->device);
  const bool gas = s->gas;
  const int n = s->numel, mu = s->o.matriz_u, mpc = s->o.matriz_pc;
  const fvc_cell_mesh *m = &s->m;
  cudaStream_t st = s->stream;
  int32_t rc;
  for (int it = 0; it < nit; ++it) {
    int solver_its[4] = {0, 0, 0, 0};
    // guess; gradients of u1, u2 (momentum ghost rules) and p
    fvc::split_w<<<fvc::g(n), fvc::kT, 0, st>>>(n, s->w, s->u1, s->u2);
    fvc::count_launch();
    if ((rc = fvc_cells_gradient(m, 1, 1, s->u1, s->gu1, st)) != FVC_OK) return rc;
    if ((rc = fvc_cells_gradient(m, 1, 2, s->u2, s->gu2, st)) != FVC_OK) return rc;
    if ((rc = fvc_cells_divergence(n, s->div, s->gu1, s->gu2, st)) != FVC_OK) return rc;
    // the pressure's ghost rules: incompressible, or the ideal-gas cell's (p)
    if ((rc = fvc_cells_gradient(m, gas ? 3 : 2, 3, s->p, s->gp, st)) != FVC_OK) return rc;
    // momentum systems (u0 = p), time term, cell residuals
    if (gas)
      rc = fvc_cells_momentum_ideal_gas(m, 1, 1, s->u1, s->p, s->w, s->gu1, s->gu2, s->gp, s->ro,
                                        s->div, s->grav[0], s->grav[1], s->o.dt, s->o.bs,
                                        s->o.under_u, s->o.simple_c, mu, s->ia_u, s->ja_u,
                                        s->ad1, s->au1, s->b1, s->im, s->d, s->rc1, st);
    else
      rc = fvc_cells_momentum(m, 1, 1, s->u1, s->p, s->w, s->gu1, s->gu2, s->gp, s->o.dt,
                              s->o.bs, s->o.under_u, s->o.simple_c, mu, s->ia_u, s->ja_u, s->ad1,
                              s->au1, s->b1, s->im, s->d, s->rc1, st);
    if (rc != FVC_OK) return rc;
    fvc::add_time_term<<<fvc::g(n), fvc::kT, 0, st>>>(n, s->num, s->b1, s->b10, s->rc1);
    fvc::count_launch();
    if (gas)
      rc = fvc_cells_momentum_ideal_gas(m, 2, 1, s->u2, s->p, s->w, s->gu2, s->gu1, s->gp, s->ro,
                                        s->div, s->grav[0], s->grav[1], s->o.dt, s->o.bs,
                                        s->o.under_u, s->o.simple_c, mu, s->ia_u, s->ja_u,
                                        s->ad2, s->au2, s->b2, s->im, s->d, s->rc2, st);
    else
      rc = fvc_cells_momentum(m, 2, 1, s->u2, s->p, s->w, s->gu2, s->gu1, s->gp, s->o.dt,
                              s->o.bs, s->o.under_u, s->o.simple_c, mu, s->ia_u, s->ja_u, s->ad2,
                              s->au2, s->b2, s->im, s->d, s->rc2, st);
    if (rc != FVC_OK) return rc;
    fvc::add_time_term<<<fvc::g(n), fvc::kT, 0, st>>>(n, s->num, s->b2, s->b20, s->rc2);
    fvc::count_launch();
    fvc::self_dots<<<2, fvc::kT, 0, st>>>(n, s->b1, s->b2, s->b2, s->dots);
    fvc::count_launch();
    cudaMemcpyAsync(s->h_dots, s->dots, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return FVC_ERR_CUDA;
    const bool solve1 = s->h_dots[0] >= 1.0e-32, solve2 = s->h_dots[1] >= 1.0e-32;
    if (solve1 && (rc = solve(s, s->ctx_u, s->o.code_u, s->ad1, s->au1, s->b1, s->u1,
                              s->o.tol_u, &solver_its[0], "u1")) != FVC_OK)
      return rc;
    if (solve2 && (rc = solve(s, s->ctx_u, s->o.code_u, s->ad2, s->au2, s->b2, s->u2,
                              s->o.tol_u, &solver_its[1], "u2")) != FVC_OK)
      return rc;
    // updateVel, p' system and the residual norms
    fvc::join_w<<<fvc::g(n), fvc::kT, 0, st>>>(n, s->wp, s->u1, s->u2);
    fvc::count_launch();
    if (gas)
      rc = fvc_cells_pressure_correction_ideal_gas(m, s->wp, s->d, s->p, s->gp, s->ro,
                                                   s->o.int_vel, s->o.dt, s->o.bs, mpc, s->ia_pc,
                                                   s->ja_pc, s->adp, s->aup, s->bp, s->rcp, st);
    else
      rc = fvc_cells_pressure_correction(m, s->wp, s->d, s->p, s->gp, s->o.int_vel, mpc,
                                         s->ia_pc, s->ja_pc, s->adp, s->aup, s->bp, s->rcp, st);
    if (rc != FVC_OK) return rc;
    fvc::self_dots<<<3, fvc::kT, 0, st>>>(n, s->rc1, s->rc2, s->rcp, s->dots);
    fvc::count_launch();
    cudaMemcpyAsync(s->h_dots, s->dots, 3 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return FVC_ERR_CUDA;
    const double r1 = std::sqrt(s->h_dots[0]), r2 = std::sqrt(s->h_dots[1]);
    const double rpc = std::sqrt(s->h_dots[2]);
    if (rpc >= 1.0e-32) {
      if ((rc = solve(s, s->ctx_pc, s->o.code_pc, s->adp, s->aup, s->bp, s->pc, s->o.tol_pc,
                      &solver_its[2], "p'")) != FVC_OK)
        return rc;
      if ((rc = fvc_cells_gradient(m, gas ? 3 : 2, 2, s->pc, s->gpc, st)) != FVC_OK) return rc;
      if ((rc = fvc_cells_simple_update(n, s->w, s->p, s->u1, s->u2, s->pc, s->gpc, s->d,
                                        s->o.under_pc, st)) != FVC_OK)
        return rc;
    }
    double re = 0.0;
    if (gas) {  // energy (src/Simple.f:647-710)
      if ((rc = fvc_cells_energy_gradient(m, 3, s->pedge_e, s->sedge_e, s->en, s->ge, st)) !=
          FVC_OK)
        return rc;
      if ((rc = fvc_cells_energy(m, 3, 1, s->pedge_e, s->sedge_e, s->en, s->en, s->ro, s->w,
                                 s->ge, s->o.dt, s->o.bs, 1, s->ia_e, s->ja_e, s->ade, s->aue,
                                 s->be, s->rce, st)) != FVC_OK)
        return rc;
      fvc::add_time_term<<<fvc::g(n), fvc::kT, 0, st>>>(n, s->num, s->be, s->be0, s->rce);
      fvc::count_launch();
      fvc::self_dots<<<2, fvc::kT, 0, st>>>(n, s->be, s->rce, s->rce, s->dots);
      fvc::count_launch();
      cudaMemcpyAsync(s->h_dots, s->dots, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
      if (cudaStreamSynchronize(st) != cudaSuccess) return FVC_ERR_CUDA;
      re = std::sqrt(s->h_dots[0]);
      if (re >= 1.0e-32) {
        re = std::sqrt(s->h_dots[1]);
        if ((rc = solve(s, s->ctx_e, 2, s->ade, s->aue, s->be, s->en, s->o.tol_u,
                        &solver_its[3], "energy")) != FVC_OK)
          return rc;
        if ((rc = fvc_cells_enthalpy_temperature(n, s->en, s->temp, s->cp, s->tref, 1, st)) !=
                FVC_OK ||
            (rc = fvc_cells_ideal_gas_density(n, s->ro, s->temp, 1, 3, 1.0, 1.0, st)) != FVC_OK)
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

}  // namespace

extern "C" {

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
