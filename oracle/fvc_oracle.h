/*
 * fvc_oracle.h -- CPU restatement of the fortranFVCell linear-solver hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GPU
 * product (libfvcgpu) and the timed CPU baseline in bench.py.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
 * product never links, calls or falls back to it.
 *
 * Every routine restates one Fortran routine of the reference with the same
 * loop order and 1-based index semantics, so integer outputs (RCM permutation,
 * CSR ia/ja, ELL ja) can be diffed verbatim and floating-point outputs follow
 * the same summation order.  All integer arrays use Fortran 1-based values;
 * the C arrays themselves are 0-based storage of those values.
 *
 * Pinning: the reference ships no golden outputs and no Fortran compiler is
 * available, so this restatement is pinned only by the reference's own
 * known-answer test (dot(i, 2i) = 2 n(n+1)(2n+1)/6, src/BenchMark.f:444-485)
 * and by hand-derived cases (tests/golden/).  Status: partially pinned.
 */
#ifndef FVC_ORACLE_H
#define FVC_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- mesh -> equation graph (host, once per mesh) ---------------------- */
/* src/Adjacency.f:1-94  (ix is ix(nen+1,numel): nen nodes + material) */
void oref_adjtria3(const int32_t *ix, int32_t *nodcon, int32_t *nelcon,
                   int32_t nnode, int32_t numel, int32_t nen, int32_t *nedge);
/* src/Adjacency.f:95-189 */
void oref_adjquad4(const int32_t *ix, int32_t *nodcon, int32_t *nelcon,
                   int32_t nnode, int32_t numel, int32_t nen, int32_t *nedge);
/* adjquad4's algorithm generalised to mixed triangle/quad meshes
 * (ix(ld,numel) with 0 in unused node slots); no reference counterpart */
void oref_adjacency_mixed(const int32_t *ix, int32_t ld, int32_t *nodcon,
                          int32_t *nelcon, int32_t nnode, int32_t numel,
                          int32_t nshared);
/* src/Reord.f:6-52 (alf = freord); iperm(old) = new */
void oref_reord(const int32_t *viz, int32_t *iperm, int32_t numel,
                int32_t nshared, int32_t alf);
/* src/Numeq.f:4-25 */
void oref_numeq(int32_t *id, const int32_t *num, const int32_t *elconn,
                int32_t numel, int32_t nshared, int32_t *neq);
/* src/Csr.f:21-55 */
void oref_csria(int32_t *ia, const int32_t *id, int32_t neq, int32_t nshared,
                int32_t *nad, int32_t upper, int32_t lower, int32_t diag);
/* src/Csr.f:76-110 */
void oref_csrja(const int32_t *ia, int32_t *ja, const int32_t *id, int32_t neq,
                int32_t nshared, int32_t upper, int32_t lower, int32_t diag);
/* src/Graph.f:45-93 */
void oref_sortgraph(const int32_t *ia, int32_t *ja, int32_t neq);
/* src/EllPack.f:19-42 */
void oref_ellpackja(int32_t *ifellpack, int32_t *ja, const int32_t *id,
                    int32_t neq, int32_t *nad, int32_t nshared);
/* src/Csr.f:245-272 (band only, no printing) */
int32_t oref_banda_csr(const int32_t *ia, const int32_t *ja, int32_t neq);
/* src/Datastruct.f:27-179 structure part: fills ia/ja for matriz 1..4.
 * ia must hold neq+1 (or 2 for ELL) and ja the size returned by the
 * first call with ja == NULL.  Returns nad. */
int32_t oref_datastruc(const int32_t *id, int32_t *ia, int32_t *ja, int32_t neq,
                       int32_t nshared, int32_t matriz, int32_t unsym);

/* ---- global scatter of one cell's coefficients ------------------------- */
/* src/Assbly.f:32-54 -> src/Csr.f:142-227 / src/EllPack.f:68-93.
 * la(nshared+1) local coefficients (la(nshared+1) = diagonal),
 * ld(nshared+1) equation numbers (ld(nshared+1) = this row; <=0 = none). */
void oref_assbly(double *ad, double *au, double *al, double *f,
                 const int32_t *ia, const int32_t *ja, const double *la,
                 double p, const int32_t *ld, int32_t nshared, int32_t cod,
                 int32_t unsym, int32_t forces, int32_t matrix);

/* Pressure-correction coefficients of one mesh (src/Pform.f:277-432 ->
 * src/Celllib.f:695-794, :596-655 -> src/CellibPressure.f:476-572 ->
 * src/Assbly.f).  ix(ld,numel) 1-based nodes (0 = unused slot),
 * nelcon(nshared,numel), num(numel), kprop(numel) = k(2,cell),
 * dsim(2,numel) = SIMPLE d; writes ad(neq) and au (CSRD slots or ELL). */
void oref_pform_pressure(const double *coor, int32_t nnode, const int32_t *ix,
                         int32_t ld, int32_t numel, int32_t nshared,
                         const int32_t *nelcon, const int32_t *num,
                         const double *kprop, const double *dsim,
                         int32_t pin_cell, int32_t int_vel, int32_t matriz,
                         int32_t unsym, const int32_t *ia, const int32_t *ja,
                         double *ad, double *au);

/* ---- SpMV + BLAS-1 (src/Matvec.f) -------------------------------------- */
void oref_matvec_csrd(const double *ad, const double *a, const double *dum,
                      const double *x, double *y, const int32_t *ia,
                      const int32_t *ja, int32_t neq);
void oref_matvec_csr(const double *a, const double *d1, const double *d2,
                     const double *x, double *y, const int32_t *ia,
                     const int32_t *ja, int32_t neq);
void oref_matvec_csrc(const double *ad, const double *au, const double *al,
                      const double *x, double *y, const int32_t *ia,
                      const int32_t *ja, int32_t neq);
void oref_matvec_csrc_sym(const double *ad, const double *dum, const double *al,
                          const double *x, double *y, const int32_t *ia,
                          const int32_t *ja, int32_t neq);
void oref_matvec_csrd_sym(const double *ad, const double *dum, const double *al,
                          const double *x, double *y, const int32_t *ia,
                          const int32_t *ja, int32_t neq);
void oref_matvec_ellpack(const double *ad, const double *a, const double *dum,
                         const double *x, double *y, const int32_t *nl,
                         const int32_t *ja, int32_t neq);
double oref_dot(const double *a, const double *b, int32_t n);

/* ---- Krylov solvers ---------------------------------------------------- */
enum { OREF_OK = 0, OREF_NOCONV = 1, OREF_UNSUPPORTED = 2 };

typedef struct {
  int32_t iterations;   /* j at exit (PCG/BiCGSTAB) or cycles l (GMRES) */
  int32_t inner_its;    /* GMRES total inner iterations (nit) */
  double energy;        /* x.Ax (PCG/BiCGSTAB) or x.b (GMRES) */
  double conv;          /* the stopping threshold */
  double final_crit;    /* the quantity compared against conv at exit */
  int32_t status;
} oref_stats;

/* Solver.f:28-346 dispatch.  omp_threads <= 0 selects the sequential
 * routines (openmpSolver = .false.); > 0 the *_omp routines with that many
 * threads (openmpSolver = .true., nThreadsSolver = omp_threads).
 * Like the reference, b is clobbered.  Non-convergence returns OREF_NOCONV
 * (the reference prints a warning and executes STOP). */
int32_t oref_solver(double *ad, double *au, double *al, double *x, double *b,
                    const int32_t *iax, const int32_t *ja, int32_t neq,
                    int32_t nad, int32_t unsym, double tol, int32_t maxit,
                    int32_t code, int32_t matriz, int32_t omp_threads,
                    oref_stats *st);

/* Iterativos_omp.f:30-127 pcg_omp with matvec_csrd_omp / matvec_ellpack_omp
 * and dot_ompL4, timed as the CPU baseline.  Runs at most maxit iterations
 * and reports (does not stop) non-convergence.  stop_rule 0: the
 * reference's test on sqrt|r.z|; 1: ||r||2 < tol ||b||2 (the GPU solves'
 * fvc_opts.stop_rule = 1), one extra dot_ompL4 per iteration. */
int32_t oref_pcg_omp_sample(double *ad, double *au, double *al, double *x,
                            double *b, const int32_t *iax, const int32_t *ja,
                            int32_t neq, int32_t nad, double tol, int32_t maxit,
                            int32_t matriz, int32_t nthreads, int32_t init,
                            int32_t stop_rule, oref_stats *st);

/* src/Iterativos.f:450-462 */
double oref_smachn(void);
/* src/Solver.f:368-391 */
void oref_getres(double *u, double *x, const int32_t *num, int32_t neq,
                 int32_t numel, int32_t flag);

#ifdef __cplusplus
}
#endif

/* SIMPLE outer-loop cells (fvc_oracle_simple.c).  Arrays follow the
 * reference's Fortran layouts: coor(2,nnode), ix(ld,numel) with the
 * material in row ld, nelcon(nshared,numel), pedge(nshared+1,numel),
 * sedge(3,nshared+1,numel), e(10,nmat), 2-vectors (2,numel), iM(4,numel). */
int32_t oref_gform(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                   int32_t nshared, const int32_t *nelcon, const int32_t *pedge,
                   const double *sedge, int32_t kind, int32_t comp, const double *u,
                   double *grad);
int32_t oref_pform_momentum(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                            int32_t nshared, const int32_t *nelcon, const int32_t *num,
                            const int32_t *pedge, const double *sedge, const double *e,
                            int32_t comp, int32_t iws, const double *u, const double *u0,
                            const double *w, const double *g_own, const double *g_oth,
                            const double *gradp, double dt, int32_t bs, double under_u,
                            int32_t simple_c, int32_t matriz, int32_t unsym, const int32_t *ia,
                            const int32_t *ja, double *ad, double *au, double *b, double *im,
                            double *d, double *rescell);
int32_t oref_pform_pc(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                      int32_t nshared, const int32_t *nelcon, const int32_t *num,
                      const int32_t *pedge, const double *sedge, const double *e,
                      const double *w, const double *d, const double *p,
                      const double *gradp, int32_t intvel, int32_t matriz, int32_t unsym,
                      const int32_t *ia, const int32_t *ja, double *ad, double *au, double *b,
                      double *rescell);
void oref_simple_update(double *w, double *pre, const double *u1, const double *u2,
                        const double *prec, const double *gradpc, const double *d,
                        int32_t numel, double under_pc);
void oref_divergente(double *div, const double *gu1, const double *gu2, int32_t numel);

/* Ideal-gas momentum cell cell_si_eb_idg_ggl (src/CellibSimple.f:54-377):
 * the arguments of oref_pform_momentum plus ro(3,numel) densities, div(numel)
 * the velocity divergence and grav[2] the gravity vector. */
int32_t oref_pform_momentum_idg(const double *coor, const int32_t *ix, int32_t ld,
                                int32_t numel, int32_t nshared, const int32_t *nelcon,
                                const int32_t *num, const int32_t *pedge, const double *sedge,
                                const double *e, int32_t comp, int32_t iws, const double *u,
                                const double *u0, const double *w, const double *g_own,
                                const double *g_oth, const double *gradp, const double *ro,
                                const double *div, const double *grav, double dt, int32_t bs,
                                double under_u, int32_t simple_c, int32_t matriz, int32_t unsym,
                                const int32_t *ia, const int32_t *ja, double *ad, double *au,
                                double *b, double *im, double *d, double *rescell);

/* Ideal-gas pressure correction (cell_si_p_idg_ggl iws 1) and the property
 * sweeps EnthalpyForTemp / idealGas (src/IdealGas.f). */
int32_t oref_pform_pc_idg(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                          int32_t nshared, const int32_t *nelcon, const int32_t *num,
                          const int32_t *pedge, const double *sedge, const double *e,
                          const double *w, const double *d, const double *p,
                          const double *gradp, const double *ro, int32_t intvel, double dt,
                          int32_t bs, int32_t matriz, int32_t unsym, const int32_t *ia,
                          const int32_t *ja, double *ad, double *au, double *b,
                          double *rescell);
void oref_enthalpy_temp(double *h, double *t, const double *e, int32_t numel, int32_t to_temp);
void oref_ideal_gas(double *ro, const double *temp, int32_t numel, int32_t celsius, int32_t row,
                    double pressure_ratio, double under_ro);

/* Energy / scalar transport cells (src/CellibTrans.f): lib 3 the ideal-gas
 * enthalpy cell, lib 4 the transport cell.  pedge and sedge here are the
 * scalar's (nshared+1, numel) arrays; ro(3, numel) the densities. */
int32_t oref_gform_energy(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                          int32_t nshared, const int32_t *nelcon, const int32_t *pedge,
                          const double *sedge, const double *e, int32_t lib, const double *u,
                          double *grad);
int32_t oref_pform_energy(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                          int32_t nshared, const int32_t *nelcon, const int32_t *num,
                          const int32_t *pedge, const double *sedge, const double *e,
                          int32_t lib, int32_t iws, const double *u, const double *u0,
                          const double *ro, const double *w, const double *grad, double dt,
                          int32_t bs, int32_t matriz, int32_t unsym, const int32_t *ia,
                          const int32_t *ja, double *ad, double *au, double *b, double *rescell);

#endif
