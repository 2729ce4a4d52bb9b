/*
 * fvc_oracle_simple.c -- CPU restatement of the cell routines of the
 * isothermal SIMPLE outer iteration of fortranFVCell.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the GPU assembly and
 * update kernels of libfvcgpu.  The product never links or calls this file.
 *
 * Restated, statement for statement (same operation order, no FMA
 * contraction: the Makefile builds with -ffp-contract=off):
 *   pform gather                 src/Pform.f:65-436
 *   gform                        src/Pform.f:466-646
 *   cellGeom2D, vectorKm2d       src/Celllib.f:695-794, :596-655
 *   areacell (tri / quad)        src/Celllib.f:282-358, :509-522
 *   limit                        src/Celllib.f:370-456
 *   cell_si_eb_i_ggl iws1=1,2,3  src/CellibSimple.f:591-940
 *   cell_si_eb_idg_ggl iws1=1,3  src/CellibSimple.f:54-377 (ideal gas, buoyancy)
 *   cellVel (intVel 1, 2, 5)     src/CellibSimple.f:1947-2073
 *   cell_si_p_i_ggl iws=1,2      src/CellibPressure.f:390-620
 *   simpleUpdate, divergente     src/Simple.f:871-910, :1070-1078
 *   cell_e_eb_idg_ggl iws 1,2,4  src/CellibTrans.f:39-349 (ideal-gas enthalpy)
 *   cell_t_eb_ggl iws 1,2,4      src/CellibTrans.f:390-655 (scalar transport)
 *   cell_si_p_idg_ggl iws 1,2    src/CellibPressure.f:43-246 (ideal-gas p')
 *   EnthalpyForTemp, idealGas    src/IdealGas.f:20-91,148-155
 * Meshes may mix triangles and quadrilaterals: a cell's loops run over its
 * own sides (for single-type meshes this is the reference's nshared).
 * Parity: restatement only (no Fortran compiler exists to run the
 * reference).
 */
#include "fvc_oracle.h"

#include <math.h>
#include <string.h>

#define F1(a, i) ((a)[(i)-1])
#define F2(a, d1, i, j) ((a)[((i)-1) + (size_t)((j)-1) * (size_t)(d1)])
#define F3(a, d1, d2, i, j, k) \
  ((a)[((i)-1) + (size_t)(d1) * (((j)-1) + (size_t)(d2) * (size_t)((k)-1))])

enum { MS = 4 };

/* The local molecule of pform/gform: cell nel (local index ns+1 -> slot
 * MS) and its face neighbours (local 1..ns -> slots 0..ns-1). */
typedef struct {
  int32_t nel, ns;
  int32_t viz[MS];
  int32_t nsl[MS + 1];
  double x[2][MS][MS + 1]; /* x(k, vertex l, local cell j) */
} Stencil;

/* cellGeom2D + vectorKm2d outputs for the central cell. */
typedef struct {
  double xc[2][MS + 1], mksi[MS], meta[MS], ksi[2][MS], n[2][MS], xm[2][MS];
  double df[2][MS], ca[MS], area;
  double xcg[2][MS], km[2][MS], mksif[MS];
} Geom;

static int32_t nsides(const int32_t *ix, int32_t ld, int32_t c, int32_t nshared) {
  int32_t s = 0;
  for (int32_t i = 1; i <= nshared; ++i)
    if (F2(ix, ld, i, c) > 0) ++s;
  return s;
}

static void gather(Stencil *S, const double *coor, const int32_t *ix, int32_t ld,
                   int32_t nshared, const int32_t *nelcon, int32_t nel) {
  S->nel = nel;
  S->ns = nsides(ix, ld, nel, nshared);
  for (int32_t j = 1; j <= nshared; ++j) {
    int32_t v = F2(nelcon, nshared, j, nel);
    S->viz[j - 1] = v;
    if (v > 0) {
      S->nsl[j - 1] = nsides(ix, ld, v, nshared);
      for (int32_t i = 1; i <= S->nsl[j - 1]; ++i) {
        int32_t no = F2(ix, ld, i, v);
        S->x[0][i - 1][j - 1] = F2(coor, 2, 1, no);
        S->x[1][i - 1][j - 1] = F2(coor, 2, 2, no);
      }
    }
  }
  S->nsl[MS] = S->ns;
  for (int32_t i = 1; i <= S->ns; ++i) {
    int32_t no = F2(ix, ld, i, nel);
    S->x[0][i - 1][MS] = F2(coor, 2, 1, no);
    S->x[1][i - 1][MS] = F2(coor, 2, 2, no);
  }
}

/* 0.5 |v1 x v2| with zero third components, as vet + dot_local compute it. */
static double half_cross(double a1, double a2, double b1, double b2) {
  const double c1 = a2 * 0.0 - 0.0 * b2;
  const double c2 = 0.0 * b1 - a1 * 0.0;
  const double c3 = a1 * b2 - a2 * b1;
  const double d = ((0.0 + c1 * c1) + c2 * c2) + c3 * c3;
  return 0.5 * sqrt(d);
}

/* areacell: eta(1:2, 1:ns) edge vectors (Celllib.f:282-358). */
static double areacell(const double eta[2][MS], int32_t ns) {
  if (ns == 3) return half_cross(eta[0][0], eta[1][0], eta[0][1], eta[1][1]);
  double a = half_cross(eta[0][0], eta[1][0], eta[0][1], eta[1][1]);
  a = a + half_cross(eta[0][2], eta[1][2], eta[0][3], eta[1][3]);
  a = a + half_cross(eta[0][0], eta[1][0], eta[0][3], eta[1][3]);
  a = a + half_cross(eta[0][1], eta[1][1], eta[0][2], eta[1][2]);
  return 0.5 * a;
}

static void geom(Geom *G, const Stencil *S) {
  const int32_t ns = S->ns;
  for (int32_t i = 0; i < MS; ++i) {
    G->mksi[i] = 0.0;
    G->meta[i] = 0.0;
    G->ksi[0][i] = G->ksi[1][i] = 0.0;
  }
  /* centroids: the central cell and the existing neighbours */
  for (int32_t i = 1; i <= MS + 1; ++i) {
    const int32_t slot = (i == MS + 1) ? MS : i - 1;
    if (slot < MS && (slot >= ns || S->viz[slot] <= 0)) continue;
    for (int32_t j = 1; j <= 2; ++j) {
      double s = 0.0;
      for (int32_t l = 1; l <= S->nsl[slot]; ++l) s = s + S->x[j - 1][l - 1][slot];
      G->xc[j - 1][slot] = (1.0 / S->nsl[slot]) * s;
    }
  }
  double eta[2][MS];
  for (int32_t l = 1; l <= ns; ++l) {
    const int32_t l2 = (l % ns) + 1;
    eta[0][l - 1] = S->x[0][l2 - 1][MS] - S->x[0][l - 1][MS];
    eta[1][l - 1] = S->x[1][l2 - 1][MS] - S->x[1][l - 1][MS];
  }
  G->area = areacell(eta, ns);
  for (int32_t i = 1; i <= ns; ++i) {
    if (S->viz[i - 1] > 0) {
      for (int32_t j = 1; j <= 2; ++j) {
        G->ksi[j - 1][i - 1] = G->xc[j - 1][i - 1] - G->xc[j - 1][MS];
        G->mksi[i - 1] = G->ksi[j - 1][i - 1] * G->ksi[j - 1][i - 1] + G->mksi[i - 1];
      }
      G->mksi[i - 1] = sqrt(G->mksi[i - 1]);
    }
  }
  for (int32_t i = 1; i <= ns; ++i) {
    for (int32_t j = 1; j <= 2; ++j)
      G->meta[i - 1] = G->meta[i - 1] + eta[j - 1][i - 1] * eta[j - 1][i - 1];
    G->meta[i - 1] = sqrt(G->meta[i - 1]);
  }
  for (int32_t j = 1; j <= 2; ++j)
    for (int32_t i = 1; i <= ns; ++i) {
      eta[j - 1][i - 1] = eta[j - 1][i - 1] / G->meta[i - 1];
      if (S->viz[i - 1] > 0) G->ksi[j - 1][i - 1] = G->ksi[j - 1][i - 1] / G->mksi[i - 1];
    }
  for (int32_t l = 1; l <= ns; ++l) {
    G->n[0][l - 1] = eta[1][l - 1];
    G->n[1][l - 1] = -eta[0][l - 1];
  }
  for (int32_t i = 1; i <= ns; ++i) {
    const int32_t i2 = (i % ns) + 1;
    G->xm[0][i - 1] = 0.5 * (S->x[0][i2 - 1][MS] + S->x[0][i - 1][MS]);
    G->xm[1][i - 1] = 0.5 * (S->x[1][i2 - 1][MS] + S->x[1][i - 1][MS]);
    G->df[0][i - 1] = G->xm[0][i - 1] - G->xc[0][MS];
    G->df[1][i - 1] = G->xm[1][i - 1] - G->xc[1][MS];
    G->ca[i - 1] = G->df[0][i - 1] * G->n[0][i - 1] + G->df[1][i - 1] * G->n[1][i - 1];
  }
  /* ghost centroids of boundary faces (both cell libraries) */
  for (int32_t i = 1; i <= ns; ++i) {
    if (S->viz[i - 1] < 0) {
      for (int32_t j = 1; j <= 2; ++j)
        G->xcg[j - 1][i - 1] = G->xc[j - 1][MS] + 2.0 * G->ca[i - 1] * G->n[j - 1][i - 1];
    } else {
      for (int32_t j = 1; j <= 2; ++j) G->xcg[j - 1][i - 1] = G->xc[j - 1][i - 1];
    }
  }
  /* vectorKm2d */
  for (int32_t i = 1; i <= ns; ++i) {
    const int32_t no1 = i, no2 = (i % ns) + 1;
    const double a1 = G->xcg[1][i - 1] - G->xc[1][MS];
    const double b1 = G->xc[0][MS] - G->xcg[0][i - 1];
    const double c1 = G->xcg[0][i - 1] * G->xc[1][MS] - G->xc[0][MS] * G->xcg[1][i - 1];
    const double a2 = S->x[1][no1 - 1][MS] - S->x[1][no2 - 1][MS];
    const double b2 = S->x[0][no2 - 1][MS] - S->x[0][no1 - 1][MS];
    const double c2 =
        S->x[0][no1 - 1][MS] * S->x[1][no2 - 1][MS] - S->x[0][no2 - 1][MS] * S->x[1][no1 - 1][MS];
    const double det = a1 * b2 - a2 * b1;
    const double m11 = (1.0 / det) * b2, m12 = -(1.0 / det) * b1;
    const double m21 = -(1.0 / det) * a2, m22 = (1.0 / det) * a1;
    const double f1 = -c1, f2 = -c2;
    const double xi1 = m11 * f1 + m12 * f2, xi2 = m21 * f1 + m22 * f2;
    G->km[0][i - 1] = G->xm[0][i - 1] - xi1;
    G->km[1][i - 1] = G->xm[1][i - 1] - xi2;
    const double k1 = xi1 - G->xc[0][MS], k2 = xi2 - G->xc[1][MS];
    G->mksif[i - 1] = sqrt(k1 * k1 + k2 * k2);
  }
}

/* limit(r, icod): Celllib.f:370-456 (codes 1-7). */
static double limit(double r, int32_t icod) {
  switch (icod) {
    case 1: return 0.0;
    case 2: return 1.0;
    case 3: return (r + fabs(r)) / (1.0 + fabs(r));
    case 4: return (r > 0.0) ? (r + r * r) / (1.0 + r * r) : 0.0;
    case 5: return fmax(0.0, fmin(r, 1.0));
    case 6: return fmax(0.0, fmin(2.0, r));
    default: {
      const double a = fmin(2.0 * r, 1.0);
      const double b = fmin(r, 2.0);
      const double c = fmax(a, b);
      return fmax(0.0, c);
    }
  }
}

/* Green-Gauss over the polygon of ghost / neighbour centroids: label 200
 * of cell_si_eb_i_ggl (CellibSimple.f:895-926) and cell_si_p_i_ggl
 * (CellibPressure.f:577-612). */
static void green_gauss(const Geom *G, int32_t ns, const double *ug, double *g1, double *g2) {
  double eta[2][MS], n[2][MS];
  for (int32_t i = 1; i <= 2; ++i)
    for (int32_t l = 1; l <= ns; ++l) {
      const int32_t s1 = l, s2 = (l % ns) + 1;
      eta[i - 1][l - 1] = G->xcg[i - 1][s2 - 1] - G->xcg[i - 1][s1 - 1];
    }
  for (int32_t l = 1; l <= ns; ++l) {
    n[0][l - 1] = eta[1][l - 1];
    n[1][l - 1] = -eta[0][l - 1];
  }
  const double area = areacell(eta, ns);
  double um[MS];
  for (int32_t l = 1; l <= ns; ++l) {
    const int32_t s1 = l, s2 = (l % ns) + 1;
    um[l - 1] = 0.5 * (ug[s2 - 1] + ug[s1 - 1]);
  }
  double a = 0.0, b = 0.0;
  for (int32_t i = 1; i <= ns; ++i) {
    const double uf = um[i - 1];
    a = a + uf * n[0][i - 1];
    b = b + uf * n[1][i - 1];
  }
  *g1 = a / area;
  *g2 = b / area;
}

int32_t oref_gform(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                   int32_t nshared, const int32_t *nelcon, const int32_t *pedge,
                   const double *sedge, int32_t kind, int32_t comp, const double *u,
                   double *grad) {
  const int32_t ldp = nshared + 1;
  for (int32_t nel = 1; nel <= numel; ++nel) {
    Stencil S;
    Geom G;
    gather(&S, coor, ix, ld, nshared, nelcon, nel);
    geom(&G, &S);
    const double uP = F1(u, nel);
    const double go1 = F2(grad, 2, 1, nel), go2 = F2(grad, 2, 2, nel);
    double ug[MS];
    for (int32_t i = 1; i <= S.ns; ++i) {
      const int32_t v = S.viz[i - 1];
      if (v > 0) {
        ug[i - 1] = F1(u, v);
        continue;
      }
      const int32_t pe = F2(pedge, ldp, i, nel);
      if (kind == 1) { /* momentum (CellibSimple.f:655-669) */
        if (pe == 0)
          ug[i - 1] = -uP;
        else if (pe == 1 || pe == 2)
          ug[i - 1] = F3(sedge, 3, ldp, comp, i, nel);
        else if (pe == 3 || pe == 4)
          ug[i - 1] = uP;
        else
          return -1; /* the reference leaves the ghost value undefined */
      } else if (kind == 3) { /* ideal-gas pressure (CellibPressure.f:115-129):
                                comp 2 = p' (gform iws1 2), comp 3 = p (iws1 3) */
        if (pe == 3) {
          ug[i - 1] = (comp == 2) ? 0.0 : F3(sedge, 3, ldp, 3, i, nel);
        } else {
          const double gama = 2.0 * G.ca[i - 1];
          ug[i - 1] = uP + gama * (go1 * G.n[0][i - 1] + go2 * G.n[1][i - 1]);
        }
      } else {       /* pressure, gform's iws = 2 (CellibPressure.f:449-462) */
        if (pe == 3) {
          ug[i - 1] = 0.0;
        } else if (pe == 6) {
          ug[i - 1] = uP;
        } else {
          const double gama = 2.0 * G.ca[i - 1];
          ug[i - 1] = uP + gama * (go1 * G.n[0][i - 1] + go2 * G.n[1][i - 1]);
        }
      }
    }
    double g1, g2;
    green_gauss(&G, S.ns, ug, &g1, &g2);
    F2(grad, 2, 1, nel) = g1;
    F2(grad, 2, 2, nel) = g2;
  }
  return 0;
}

/* Material property k(i) of cell c: e(i, ix(ld, c)). */
#define PROP(e, ix, ld, c, i) F2(e, 10, i, F2(ix, ld, ld, c))

/* The momentum cells: cell_si_eb_i_ggl (incompressible, idg = 0) and
 * cell_si_eb_idg_ggl (ideal gas, idg = 1; CellibSimple.f:54-536).  The
 * ideal-gas cell takes the density from ro(3,*) (row 3 the current iterate,
 * rows 1-2 the time levels) wherever the incompressible one uses the
 * material's e(2), adds the -2/3 mu div(w) terms, the buoyancy source
 * (ro - e(2)) g A and has no fixed-velocity pin (pedge -2). */
static int32_t pform_momentum_cells(const double *coor, const int32_t *ix, int32_t ld,
                                    int32_t numel, int32_t nshared, const int32_t *nelcon,
                                    const int32_t *num, const int32_t *pedge, const double *sedge,
                                    const double *e, int32_t comp, int32_t iws, const double *u,
                                    const double *u0, const double *w, const double *g_own,
                                    const double *g_oth, const double *gradp, double dt,
                                    int32_t bs, double under_u, int32_t simple_c, int32_t matriz,
                                    int32_t unsym, const int32_t *ia, const int32_t *ja,
                                    double *ad, double *au, double *b, double *im, double *d,
                                    double *rescell, int32_t idg, const double *ro,
                                    const double *div, const double *grav) {
  const int32_t ldp = nshared + 1;
  const double ZERO = 1.0e-7, eps = 1.0e-14, cnst = 1.0e60;
  for (int32_t nel = 1; nel <= numel; ++nel) {
    Stencil S;
    Geom G;
    gather(&S, coor, ix, ld, nshared, nelcon, nel);
    geom(&G, &S);
    const int32_t ns = S.ns;
    const double viscosity = PROP(e, ix, ld, nel, 1);
    const double rhoA = PROP(e, ix, ld, nel, 2);
    const double cc = PROP(e, ix, ld, nel, 6);
    const int32_t icod = (int32_t)PROP(e, ix, ld, nel, 7);
    const double uP = F1(u, nel);
    int32_t ldl[MS + 1];
    for (int32_t i = 0; i <= MS; ++i) ldl[i] = 0;
    for (int32_t j = 1; j <= ns; ++j) ldl[j - 1] = (S.viz[j - 1] > 0) ? F1(num, S.viz[j - 1]) : 0;
    ldl[nshared] = F1(num, nel);
    double la[MS + 1];
    for (int32_t i = 0; i <= MS; ++i) la[i] = 0.0;
    if (iws == 3) { /* F = rho cc A/dt u (label 300) */
      double m = (idg ? F2(ro, 3, 2, nel) : PROP(e, ix, ld, nel, 2)) * cc * G.area / dt;
      double p = m * uP;
      m = (idg ? F2(ro, 3, 1, nel) : PROP(e, ix, ld, nel, 2)) * cc * G.area / dt;
      if (bs) p = 2 * p - 0.5 * m * F1(u0, nel);
      oref_assbly(ad, au, au, b, ia, ja, la, p, ldl, nshared, matriz, unsym, 1, 0);
      continue;
    }
    /* ideal gas: the cell's current density (specificMass) */
    const double rhoP = idg ? F2(ro, 3, 3, nel) : rhoA;
    double p = 0.0, pf = 0.0, sp = 0.0, cd = 0.0, cvc = 0.0;
    double a[MS + 1];
    for (int32_t i = 1; i <= ns; ++i) {
      const int32_t v = S.viz[i - 1];
      const double n1 = G.n[0][i - 1], n2 = G.n[1][i - 1];
      const double meta = G.meta[i - 1];
      if (v < 0) {
        const int32_t pe = F2(pedge, ldp, i, nel);
        a[i - 1] = 0.0;
        double ap = viscosity * meta;
        if (comp == 1)
          p = p + ap * (F2(g_own, 2, comp, nel) * n1 + F2(g_oth, 2, comp, nel) * n2);
        else
          p = p + ap * (F2(g_own, 2, comp, nel) * n2 + F2(g_oth, 2, comp, nel) * n1);
        if (idg) p = p - (2.0 / 3.0) * ap * F1(div, nel) * G.n[comp - 1][i - 1];
        double pface;
        if (pe == 3) {
          pface = F3(sedge, 3, ldp, 3, i, nel);
        } else {
          pface = F1(u0, nel);
          pface = pface + (F2(gradp, 2, 1, nel) * G.df[0][i - 1] +
                           F2(gradp, 2, 2, nel) * G.df[1][i - 1]);
        }
        pf = pf + pface * meta * G.n[comp - 1][i - 1];
        if (pe == 0) {
          ap = viscosity * meta / G.ca[i - 1];
          sp = sp + ap;
        } else if (pe == 1) {
          ap = viscosity * meta / G.ca[i - 1];
          sp = sp + ap;
          p = p + ap * F3(sedge, 3, ldp, comp, i, nel);
        } else if (pe == 2) {
          const double wfn = F3(sedge, 3, ldp, 1, i, nel) * n1 + F3(sedge, 3, ldp, 2, i, nel) * n2;
          const double cv = rhoA * wfn * meta;
          p = p - cv * F3(sedge, 3, ldp, comp, i, nel);
        } else if (pe == 3) {
          const double wfn = F2(w, 2, 1, nel) * n1 + F2(w, 2, 2, nel) * n2;
          if (fabs(wfn) > ZERO) {
            if (wfn > 0.0) {
              const double cv = rhoP * wfn * meta;
              sp = sp + cv;
            } else if (wfn < 0.0) {
              const double cv = rhoA * wfn * meta;
              p = p + cv * wfn;
            }
          }
        } else if (pe == 4) {
          const double wfn = F2(w, 2, 1, nel) * n1 + F2(w, 2, 2, nel) * n2;
          const double cv = rhoP * wfn * meta;
          sp = sp + cv;
        }
      } else {
        double alpha = G.mksif[i - 1] / G.mksi[i - 1];
        double kf = alpha / viscosity + (1.0 - alpha) / PROP(e, ix, ld, v, 1);
        kf = 1.0 / kf;
        const double wf1 = (1.0 - alpha) * F2(w, 2, 1, nel) + alpha * F2(w, 2, 1, v);
        const double wf2 = (1.0 - alpha) * F2(w, 2, 2, nel) + alpha * F2(w, 2, 2, v);
        double gf1 = (1.0 - alpha) * F2(g_own, 2, 1, nel) + alpha * F2(g_own, 2, 1, v);
        double gf2 = (1.0 - alpha) * F2(g_own, 2, 2, nel) + alpha * F2(g_own, 2, 2, v);
        const double k1 = G.ksi[0][i - 1], k2 = G.ksi[1][i - 1], mk = G.mksi[i - 1];
        const double nk = n1 * k1 + n2 * k2;
        const double wfn = wf1 * n1 + wf2 * n2;
        double gfk = gf1 * k1 + gf2 * k2;
        gf1 = gf1 + ((F1(u, v) - uP) / mk - gfk) * k1;
        gf2 = gf2 + ((F1(u, v) - uP) / mk - gfk) * k2;
        const double gfn = gf1 * n1 + gf2 * n2;
        gfk = gf1 * k1 + gf2 * k2;
        const double dfd = (kf * meta) / (nk * mk);
        cd = kf * meta * (gfn - gfk / nk);
        a[i - 1] = dfd;
        p = p + cd;
        const double rof =
            idg ? (1.0 - alpha) * F2(ro, 3, 3, nel) + alpha * F2(ro, 3, 3, v) : rhoA;
        const double cv = rof * wfn * meta;
        if (cv < 0.0) {
          const double du = uP - F1(u, v) + eps;
          const double gpk = F2(g_own, 2, 1, v) * (G.xc[0][MS] - G.xc[0][i - 1]) +
                             F2(g_own, 2, 2, v) * (G.xc[1][MS] - G.xc[1][i - 1]);
          alpha = G.mksif[i - 1] / G.mksi[i - 1];
          const double r = 2.0 * gpk / du - 1.0;
          cvc = (1.0 - alpha) * limit(r, icod) * du;
        } else {
          const double du = F1(u, v) - uP + eps;
          const double gpk = (F2(g_own, 2, 1, nel) * k1 + F2(g_own, 2, 2, nel) * k2) * mk;
          alpha = G.mksif[i - 1] / G.mksi[i - 1];
          const double r = 2.0 * gpk / du - 1.0;
          cvc = alpha * limit(r, icod) * du;
        }
        cvc = cvc + gf1 * G.km[0][i - 1] + gf2 * G.km[1][i - 1];
        a[i - 1] = a[i - 1] + fmax(-cv, 0.0);
        sp = sp + cv;
        p = p - cv * cvc;
        /* second-order face pressure (sPressure) */
        alpha = G.mksif[i - 1] / G.mksi[i - 1];
        const double p1 = F1(u0, nel) + F2(gradp, 2, 1, nel) * G.df[0][i - 1] +
                          F2(gradp, 2, 2, nel) * G.df[1][i - 1];
        const double p2 = F1(u0, v) + F2(gradp, 2, 1, v) * (G.xm[0][i - 1] - G.xc[0][i - 1]) +
                          F2(gradp, 2, 2, v) * (G.xm[1][i - 1] - G.xc[1][i - 1]);
        const double pface = 0.5 * (p1 + p2);
        pf = pf + pface * meta * G.n[comp - 1][i - 1];
        /* transposed viscous stress */
        alpha = G.mksif[i - 1] / G.mksi[i - 1];
        gf1 = (1.0 - alpha) * F2(g_own, 2, comp, nel) + alpha * F2(g_own, 2, comp, v);
        gf2 = (1.0 - alpha) * F2(g_oth, 2, comp, nel) + alpha * F2(g_oth, 2, comp, v);
        if (comp == 1)
          p = p + kf * meta * (gf1 * n1 + gf2 * n2);
        else
          p = p + kf * meta * (gf1 * n2 + gf2 * n1);
        if (idg) { /* -2/3 mu div(w) on the face */
          const double gdiv = (1.0 - alpha) * F1(div, nel) + alpha * F1(div, v);
          p = p - (2.0 / 3.0) * kf * gdiv * meta * G.n[comp - 1][i - 1];
        }
      }
    }
    if (!idg && F2(pedge, ldp, ldp, nel) == -2) sp = sp + cnst;
    double aP = sp;
    for (int32_t i = 1; i <= ns; ++i) aP = aP + a[i - 1];
    double m = rhoP * cc * G.area / dt;
    if (bs) m = 1.5 * m;
    aP = aP + m;
    aP = aP / under_u;
    p = p + (1 - under_u) * aP * uP;
    if (idg) /* buoyancy: (rho - rho_ref) g A, rho_ref = e(2) */
      p = p + (F2(ro, 3, 3, nel) - rhoA) * grav[comp - 1] * G.area;
    double rm = 0.0, anb = 0.0;
    for (int32_t i = 1; i <= ns; ++i) {
      rm = rm + a[i - 1] * ((S.viz[i - 1] > 0) ? F1(u, S.viz[i - 1]) : 0.0);
      anb = anb + a[i - 1];
    }
    F2(im, 4, comp, nel) = rm + p;
    F2(im, 4, comp + 2, nel) = aP;
    if (simple_c)
      F2(d, 2, comp, nel) = G.area / (aP - anb);
    else
      F2(d, 2, comp, nel) = G.area / aP;
    p = p - pf;
    rm = p + rm - aP * uP;
    F1(rescell, nel) = rm;
    for (int32_t i = 1; i <= ns; ++i) la[i - 1] = a[i - 1];
    la[nshared] = aP;
    oref_assbly(ad, au, au, b, ia, ja, la, p, ldl, nshared, matriz, unsym, 1, 1);
  }
  return 0;
}

int32_t oref_pform_momentum(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                            int32_t nshared, const int32_t *nelcon, const int32_t *num,
                            const int32_t *pedge, const double *sedge, const double *e,
                            int32_t comp, int32_t iws, const double *u, const double *u0,
                            const double *w, const double *g_own, const double *g_oth,
                            const double *gradp, double dt, int32_t bs, double under_u,
                            int32_t simple_c, int32_t matriz, int32_t unsym, const int32_t *ia,
                            const int32_t *ja, double *ad, double *au, double *b, double *im,
                            double *d, double *rescell) {
  return pform_momentum_cells(coor, ix, ld, numel, nshared, nelcon, num, pedge, sedge, e, comp,
                              iws, u, u0, w, g_own, g_oth, gradp, dt, bs, under_u, simple_c,
                              matriz, unsym, ia, ja, ad, au, b, im, d, rescell, 0, NULL, NULL,
                              NULL);
}

int32_t oref_pform_momentum_idg(const double *coor, const int32_t *ix, int32_t ld,
                                int32_t numel, int32_t nshared, const int32_t *nelcon,
                                const int32_t *num, const int32_t *pedge, const double *sedge,
                                const double *e, int32_t comp, int32_t iws, const double *u,
                                const double *u0, const double *w, const double *g_own,
                                const double *g_oth, const double *gradp, const double *ro,
                                const double *div, const double *grav, double dt, int32_t bs,
                                double under_u, int32_t simple_c, int32_t matriz, int32_t unsym,
                                const int32_t *ia, const int32_t *ja, double *ad, double *au,
                                double *b, double *im, double *d, double *rescell) {
  return pform_momentum_cells(coor, ix, ld, numel, nshared, nelcon, num, pedge, sedge, e, comp,
                              iws, u, u0, w, g_own, g_oth, gradp, dt, bs, under_u, simple_c,
                              matriz, unsym, ia, ja, ad, au, b, im, d, rescell, 1, ro, div, grav);
}

/* cellVel (CellibSimple.f:1947-2073): face flux w_f.n |f| for intVel 1, 2, 5.
 * p is the pressure field, d the momentum D field, df the face D. */
static double cell_vel(int32_t intvel, const double *w, const double *grad, const double ddf[2],
                       const Geom *G, const double *p, int32_t nel, int32_t v, int32_t i,
                       double alpha) {
  const double n1 = G->n[0][i - 1], n2 = G->n[1][i - 1];
  const double vm1 = (1 - alpha) * F2(w, 2, 1, nel) + alpha * F2(w, 2, 1, v);
  const double vm2 = (1 - alpha) * F2(w, 2, 2, nel) + alpha * F2(w, 2, 2, v);
  double wfn = vm1 * n1 + vm2 * n2;
  if (intvel == 1) return wfn * G->meta[i - 1];
  const double gf1 = (1 - alpha) * F2(grad, 2, 1, nel) + alpha * F2(grad, 2, 1, v);
  const double gf2 = (1 - alpha) * F2(grad, 2, 2, nel) + alpha * F2(grad, 2, 2, v);
  if (intvel == 2) {
    const double gfp1 = ((F1(p, v) - F1(p, nel)) / G->mksi[i - 1]);
    const double gfp2 = gf1 * G->ksi[0][i - 1] + gf2 * G->ksi[1][i - 1];
    wfn = wfn + 0.5 * (ddf[0] + ddf[1]) * (gfp2 - gfp1);
    return wfn * G->meta[i - 1];
  }
  /* 5: Ferziger-Peric */
  const double gfp1 = F1(p, v) - F1(p, nel);
  const double ks1 = G->mksi[i - 1] * G->ksi[0][i - 1];
  const double ks2 = G->mksi[i - 1] * G->ksi[1][i - 1];
  const double nk = ks1 * n1 + ks2 * n2;
  double gfp2 = gf1 * ks1 + gf2 * ks2;
  gfp2 = (gfp2 - gfp1) / nk;
  wfn = wfn + 0.5 * (ddf[0] + ddf[1]) * gfp2;
  return wfn * G->meta[i - 1];
}

int32_t oref_pform_pc(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                      int32_t nshared, const int32_t *nelcon, const int32_t *num,
                      const int32_t *pedge, const double *sedge, const double *e,
                      const double *w, const double *d, const double *p,
                      const double *gradp, int32_t intvel, int32_t matriz, int32_t unsym,
                      const int32_t *ia, const int32_t *ja, double *ad, double *au, double *b,
                      double *rescell) {
  const int32_t ldp = nshared + 1;
  const double cnst = 1.0e60;
  /* cellVel leaves the face flux undefined for intVel 3, 4 and 6 */
  if (intvel != 1 && intvel != 2 && intvel != 5) return -1;
  for (int32_t nel = 1; nel <= numel; ++nel) {
    Stencil S;
    Geom G;
    gather(&S, coor, ix, ld, nshared, nelcon, nel);
    geom(&G, &S);
    const int32_t ns = S.ns;
    const double rhoA = PROP(e, ix, ld, nel, 2);
    int32_t ldl[MS + 1];
    for (int32_t i = 0; i <= MS; ++i) ldl[i] = 0;
    for (int32_t j = 1; j <= ns; ++j) ldl[j - 1] = (S.viz[j - 1] > 0) ? F1(num, S.viz[j - 1]) : 0;
    ldl[nshared] = F1(num, nel);
    double la[MS + 1];
    for (int32_t i = 0; i <= MS; ++i) la[i] = 0.0;
    double pp = 0.0, sp = 0.0, kf = 0.0;
    for (int32_t i = 1; i <= ns; ++i) {
      const int32_t v = S.viz[i - 1];
      const double n1 = G.n[0][i - 1], n2 = G.n[1][i - 1];
      if (v < 0) {
        const int32_t pe = F2(pedge, ldp, i, nel);
        la[i - 1] = 0.0;
        if (pe == 2 || pe == 4) {
          const double wfn = F3(sedge, 3, ldp, 1, i, nel) * n1 + F3(sedge, 3, ldp, 2, i, nel) * n2;
          const double cv = rhoA * wfn * G.meta[i - 1];
          pp = pp - cv;
        } else if (pe == 3) {
          const double dd1 = F2(d, 2, 1, nel) * n1, dd2 = F2(d, 2, 2, nel) * n2;
          const double ndd = dd1 * n1 + dd2 * n2;
          const double dfd = (rhoA * ndd * G.meta[i - 1]) / G.ca[i - 1];
          sp = sp + dfd;
          const double wfn = F2(w, 2, 1, nel) * n1 + F2(w, 2, 2, nel) * n2;
          const double cv = rhoA * wfn * G.meta[i - 1];
          pp = pp - cv;
        }
      } else {
        const double alpha = G.mksif[i - 1] / G.mksi[i - 1];
        double ddf[2], ndd;
        if (intvel == 5) {
          kf = (1.0 - alpha) * PROP(e, ix, ld, nel, 2) + alpha * PROP(e, ix, ld, v, 2);
          ddf[0] = (1.0 - alpha) * F2(d, 2, 1, nel) + alpha * F2(d, 2, 1, v);
          ddf[1] = (1.0 - alpha) * F2(d, 2, 2, nel) + alpha * F2(d, 2, 2, v);
          ndd = 0.5 * (ddf[0] + ddf[1]);
        } else {
          kf = PROP(e, ix, ld, nel, 2);
          ddf[0] = (1.0 - alpha) * F2(d, 2, 1, nel) + alpha * F2(d, 2, 1, v);
          ddf[1] = (1.0 - alpha) * F2(d, 2, 2, nel) + alpha * F2(d, 2, 2, v);
          const double dd1 = ddf[0] * n1, dd2 = ddf[1] * n2;
          ndd = dd1 * n1 + dd2 * n2;
        }
        const double nk = n1 * G.ksi[0][i - 1] + n2 * G.ksi[1][i - 1];
        la[i - 1] = (kf * G.meta[i - 1] * ndd) / (nk * G.mksi[i - 1]);
        const double wfn = cell_vel(intvel, w, gradp, ddf, &G, p, nel, v, i, alpha);
        pp = pp - kf * wfn;
      }
    }
    if (F2(pedge, ldp, ldp, nel) == -1) sp = sp + cnst;
    la[nshared] = sp;
    for (int32_t i = 1; i <= ns; ++i) la[nshared] = la[nshared] + la[i - 1];
    F1(rescell, nel) = pp;
    oref_assbly(ad, au, au, b, ia, ja, la, pp, ldl, nshared, matriz, unsym, 1, 1);
  }
  return 0;
}

/* simpleUpdate (Simple.f:871-910), SIMPLE form (simpleR false). */
void oref_simple_update(double *w, double *pre, const double *u1, const double *u2,
                        const double *prec, const double *gradpc, const double *d,
                        int32_t numel, double under_pc) {
  for (int32_t i = 1; i <= numel; ++i) {
    F2(w, 2, 1, i) = F1(u1, i) - F2(d, 2, 1, i) * F2(gradpc, 2, 1, i);
    F2(w, 2, 2, i) = F1(u2, i) - F2(d, 2, 2, i) * F2(gradpc, 2, 2, i);
    F1(pre, i) = F1(pre, i) + under_pc * F1(prec, i);
  }
}

/* divergente (Simple.f:1070-1078). */
void oref_divergente(double *div, const double *gu1, const double *gu2, int32_t numel) {
  for (int32_t i = 1; i <= numel; ++i) F1(div, i) = F2(gu1, 2, 1, i) + F2(gu2, 2, 2, i);
}

/* ---- energy / scalar transport cells (src/CellibTrans.f) ---------------
 * lib 3: cell_e_eb_idg_ggl, the ideal-gas enthalpy equation
 *        (CellibTrans.f:39-349); lib 4: cell_t_eb_ggl, the scalar
 *        transport equation (CellibTrans.f:390-655).  pedge(nshared+1,*)
 *        and sedge(nshared+1,*) hold the scalar's boundary codes and values
 *        (one value per face, nst = 1); face nshared+1 carries a volume
 *        source when its code is nonzero.  ro(3,*) is the density at the
 *        time levels n-1, n and the current iterate.
 * Two of the reference's variables are declared integer, and the
 * restatement keeps that: the boundary enthalpy cEsp (T - tRef) of lib 3
 * (`enthalpia`) and the inflow density k(2) of lib 4 (`specificMassA`) are
 * truncated toward zero. */

/* Ghost value of boundary face i for the gradient (iws 2). */
static double energy_ghost(int32_t lib, int32_t pe, double sface, double uP, const Geom *G,
                           int32_t i, double go1, double go2, double cesp, double tref) {
  if (lib == 3) { /* CellibTrans.f:131-144 */
    if (pe == 2) {
      const int32_t enthalpia = (int32_t)(cesp * (sface - tref));
      return (double)enthalpia;
    }
    const double gama = 2.0 * G->ca[i - 1];
    return uP + gama * (go1 * G->n[0][i - 1] + go2 * G->n[1][i - 1]);
  }
  /* lib 4: CellibTrans.f:460-464 */
  if (pe == 2) return 2.0 * sface - uP;
  return uP;
}

/* gform for the scalar (Pform.f:466-646 with lib 3 or 4, iws 2): grad(2,*)
 * holds the previous gradient on entry (lib 3 extrapolates with it). */
int32_t oref_gform_energy(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                          int32_t nshared, const int32_t *nelcon, const int32_t *pedge,
                          const double *sedge, const double *e, int32_t lib, const double *u,
                          double *grad) {
  const int32_t ldp = nshared + 1;
  if (lib != 3 && lib != 4) return -1;
  for (int32_t nel = 1; nel <= numel; ++nel) {
    Stencil S;
    Geom G;
    gather(&S, coor, ix, ld, nshared, nelcon, nel);
    geom(&G, &S);
    const double uP = F1(u, nel);
    const double go1 = F2(grad, 2, 1, nel), go2 = F2(grad, 2, 2, nel);
    const double cesp = PROP(e, ix, ld, nel, 4), tref = PROP(e, ix, ld, nel, 5);
    double ug[MS];
    for (int32_t i = 1; i <= S.ns; ++i) {
      const int32_t v = S.viz[i - 1];
      if (v > 0)
        ug[i - 1] = F1(u, v);
      else
        ug[i - 1] = energy_ghost(lib, F2(pedge, ldp, i, nel), F2(sedge, ldp, i, nel), uP, &G, i,
                                 go1, go2, cesp, tref);
    }
    double g1, g2;
    green_gauss(&G, S.ns, ug, &g1, &g2);
    F2(grad, 2, 1, nel) = g1;
    F2(grad, 2, 2, nel) = g2;
  }
  return 0;
}

/* pform for the scalar (Pform.f:65-436 with lib 3 or 4).  iws 1: the
 * system (label 100: coefficients, b(num(c)) = p, rescell(c) = the cell
 * residual); iws 4: b(num(c)) = the time term of u and u0 plus the volume
 * source (label 400).  u0 is the level n-1 field (bs only). */
int32_t oref_pform_energy(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                          int32_t nshared, const int32_t *nelcon, const int32_t *num,
                          const int32_t *pedge, const double *sedge, const double *e,
                          int32_t lib, int32_t iws, const double *u, const double *u0,
                          const double *ro, const double *w, const double *grad, double dt,
                          int32_t bs, int32_t matriz, int32_t unsym, const int32_t *ia,
                          const int32_t *ja, double *ad, double *au, double *b, double *rescell) {
  const int32_t ldp = nshared + 1;
  const double ZERO = 1.0e-14, eps = 1.0e-14;
  if ((lib != 3 && lib != 4) || (iws != 1 && iws != 4)) return -1;
  for (int32_t nel = 1; nel <= numel; ++nel) {
    Stencil S;
    Geom G;
    gather(&S, coor, ix, ld, nshared, nelcon, nel);
    geom(&G, &S);
    const int32_t ns = S.ns;
    const double kc = PROP(e, ix, ld, nel, 3);
    const double cesp = PROP(e, ix, ld, nel, 4);
    const double tref = PROP(e, ix, ld, nel, 5);
    const double cc = PROP(e, ix, ld, nel, 6);
    const int32_t icod = (int32_t)PROP(e, ix, ld, nel, 7);
    const int32_t spec_mass = (int32_t)PROP(e, ix, ld, nel, 2); /* lib 4: integer */
    const double uP = F1(u, nel);
    int32_t ldl[MS + 1];
    for (int32_t i = 0; i <= MS; ++i) ldl[i] = 0;
    for (int32_t j = 1; j <= ns; ++j) ldl[j - 1] = (S.viz[j - 1] > 0) ? F1(num, S.viz[j - 1]) : 0;
    ldl[nshared] = F1(num, nel);
    double la[MS + 1];
    for (int32_t i = 0; i <= MS; ++i) la[i] = 0.0;
    if (iws == 4) { /* label 400 */
      double m = F2(ro, 3, 2, nel) * cc * G.area / dt;
      double p = m * uP;
      if (bs) {
        m = F2(ro, 3, 1, nel) * cc * G.area / dt;
        p = 2 * p - 0.5 * m * F1(u0, nel);
      }
      if (F2(pedge, ldp, ldp, nel) != 0) p = p + F2(sedge, ldp, ldp, nel) * G.area;
      oref_assbly(ad, au, au, b, ia, ja, la, p, ldl, nshared, matriz, unsym, 1, 0);
      continue;
    }
    const double roc = F2(ro, 3, 3, nel);
    double rof = roc; /* lib 4 keeps it as a running value across faces */
    double p = 0.0, sp = 0.0, cd = 0.0, cvc = 0.0;
    double a[MS + 1];
    for (int32_t i = 1; i <= ns; ++i) {
      const int32_t v = S.viz[i - 1];
      const double n1 = G.n[0][i - 1], n2 = G.n[1][i - 1];
      const double meta = G.meta[i - 1];
      if (v < 0) {
        const int32_t pe = F2(pedge, ldp, i, nel);
        const double sface = F2(sedge, ldp, i, nel);
        a[i - 1] = 0.0;
        const double wfn = F2(w, 2, 1, nel) * n1 + F2(w, 2, 2, nel) * n2;
        double cv = (lib == 3 ? roc : rof) * wfn * meta;
        if (pe == 0) {
          p = p + sface * meta;
        } else if (pe == 1) {
          if (lib == 3) {
            const double ap = (kc / cesp) * meta / G.ca[i - 1];
            sp = sp + ap;
            const int32_t enthalpia = (int32_t)(cesp * (sface - tref));
            p = p + ap * enthalpia;
          } else {
            const double ap = kc * meta / G.ca[i - 1];
            sp = sp + ap;
            p = p + ap * sface;
          }
        } else if (pe == 2) {
          if (lib == 3) {
            if (fabs(wfn) > ZERO) {
              if (cv < 0.0) {
                cv = PROP(e, ix, ld, nel, 2) * wfn * meta;
                const int32_t enthalpia = (int32_t)(cesp * (sface - tref));
                p = p - cv * enthalpia;
              } else {
                sp = sp + cv;
              }
            }
          } else {
            if (cv < 0.0) {
              cv = spec_mass * wfn * meta;
              p = p - cv * sface;
            } else {
              sp = sp + cv;
            }
          }
        } else if (pe == 4) {
          sp = sp + cv;
        }
      } else {
        double alpha = G.mksif[i - 1] / G.mksi[i - 1];
        double kf;
        if (lib == 3)
          kf = alpha / (kc / cesp) + (1.0 - alpha) / (PROP(e, ix, ld, v, 3) / PROP(e, ix, ld, v, 4));
        else
          kf = alpha / kc + (1.0 - alpha) / PROP(e, ix, ld, v, 3);
        kf = 1.0 / kf;
        const double wf1 = (1.0 - alpha) * F2(w, 2, 1, nel) + alpha * F2(w, 2, 1, v);
        const double wf2 = (1.0 - alpha) * F2(w, 2, 2, nel) + alpha * F2(w, 2, 2, v);
        double gf1 = (1.0 - alpha) * F2(grad, 2, 1, nel) + alpha * F2(grad, 2, 1, v);
        double gf2 = (1.0 - alpha) * F2(grad, 2, 2, nel) + alpha * F2(grad, 2, 2, v);
        const double k1 = G.ksi[0][i - 1], k2 = G.ksi[1][i - 1], mk = G.mksi[i - 1];
        const double nk = n1 * k1 + n2 * k2;
        const double wfn = wf1 * n1 + wf2 * n2;
        double gfk = gf1 * k1 + gf2 * k2;
        gf1 = gf1 + ((F1(u, v) - uP) / mk - gfk) * k1;
        gf2 = gf2 + ((F1(u, v) - uP) / mk - gfk) * k2;
        const double gfn = gf1 * n1 + gf2 * n2;
        gfk = gf1 * k1 + gf2 * k2;
        const double dfd = (kf * meta) / (nk * mk);
        cd = kf * meta * (gfn - gfk / nk);
        a[i - 1] = dfd;
        p = p + cd;
        if (lib == 3) {
          rof = (1.0 - alpha) * F2(ro, 3, 3, nel) + alpha * F2(ro, 3, 3, v);
        } else {
          if (wfn > 0.0)
            rof = F2(ro, 3, 3, nel);
          else if (wfn < 0.0)
            rof = F2(ro, 3, 3, v);
          else
            rof = (1.0 - alpha) * F2(ro, 3, 3, nel) + alpha * F2(ro, 3, 3, v);
        }
        const double cv = rof * wfn * meta;
        if (cv < 0.0) {
          const double du = uP - F1(u, v) + eps;
          const double gpk = F2(grad, 2, 1, v) * (G.xc[0][MS] - G.xc[0][i - 1]) +
                             F2(grad, 2, 2, v) * (G.xc[1][MS] - G.xc[1][i - 1]);
          alpha = G.mksif[i - 1] / G.mksi[i - 1];
          const double r = 2.0 * gpk / du - 1.0;
          cvc = (1.0 - alpha) * limit(r, icod) * du;
        } else {
          const double du = F1(u, v) - uP + eps;
          const double gpk = (F2(grad, 2, 1, nel) * k1 + F2(grad, 2, 2, nel) * k2) * mk;
          alpha = G.mksif[i - 1] / G.mksi[i - 1];
          const double r = 2.0 * gpk / du - 1.0;
          cvc = alpha * limit(r, icod) * du;
        }
        cvc = cvc + gf1 * G.km[0][i - 1] + gf2 * G.km[1][i - 1];
        a[i - 1] = a[i - 1] + fmax(-cv, 0.0);
        sp = sp + cv;
        p = p - cv * cvc;
      }
    }
    double aP = sp;
    for (int32_t i = 1; i <= ns; ++i) aP = aP + a[i - 1];
    double m = F2(ro, 3, 3, nel) * cc * G.area / dt;
    if (bs) m = 1.5 * m;
    aP = aP + m;
    /* rm = F - K u; a boundary face's coefficient is zero and its
       neighbour value counts as 0 */
    double rm = p - aP * uP;
    for (int32_t i = 1; i <= ns; ++i)
      rm = rm + a[i - 1] * ((S.viz[i - 1] > 0) ? F1(u, S.viz[i - 1]) : 0.0);
    F1(rescell, nel) = rm;
    for (int32_t i = 1; i <= ns; ++i) la[i - 1] = a[i - 1];
    la[nshared] = aP;
    oref_assbly(ad, au, au, b, ia, ja, la, p, ldl, nshared, matriz, unsym, 1, 1);
  }
  return 0;
}


/* ---- ideal gas (src/CellibPressure.f:43-389, src/IdealGas.f) ----------- */

/* Pressure correction of the ideal-gas cell cell_si_p_idg_ggl, iws = 1
 * (CellibPressure.f:122-246): face densities interpolated from ro(3,*),
 * prescribed-pressure faces (pe 3) with the D-weighted coefficient and the
 * outflow / backflow mass flux, the mass storage term -A (rho - rho_n)/dt
 * (second order with bs), rescell = |b|. */
int32_t oref_pform_pc_idg(const double *coor, const int32_t *ix, int32_t ld, int32_t numel,
                          int32_t nshared, const int32_t *nelcon, const int32_t *num,
                          const int32_t *pedge, const double *sedge, const double *e,
                          const double *w, const double *d, const double *p,
                          const double *gradp, const double *ro, int32_t intvel, double dt,
                          int32_t bs, int32_t matriz, int32_t unsym, const int32_t *ia,
                          const int32_t *ja, double *ad, double *au, double *b,
                          double *rescell) {
  const int32_t ldp = nshared + 1;
  const double cnst = 1.0e60, ZERO = 1.0e-7;
  if (intvel != 1 && intvel != 2 && intvel != 5) return -1;
  for (int32_t nel = 1; nel <= numel; ++nel) {
    Stencil S;
    Geom G;
    gather(&S, coor, ix, ld, nshared, nelcon, nel);
    geom(&G, &S);
    const int32_t ns = S.ns;
    const double rhoP = F2(ro, 3, 3, nel);
    const double rhoA = PROP(e, ix, ld, nel, 2);
    int32_t ldl[MS + 1];
    for (int32_t i = 0; i <= MS; ++i) ldl[i] = 0;
    for (int32_t j = 1; j <= ns; ++j) ldl[j - 1] = (S.viz[j - 1] > 0) ? F1(num, S.viz[j - 1]) : 0;
    ldl[nshared] = F1(num, nel);
    double la[MS + 1];
    for (int32_t i = 0; i <= MS; ++i) la[i] = 0.0;
    double pp = 0.0, sp = 0.0, kf = 0.0;
    for (int32_t i = 1; i <= ns; ++i) {
      const int32_t v = S.viz[i - 1];
      const double n1 = G.n[0][i - 1], n2 = G.n[1][i - 1];
      if (v < 0) {
        const int32_t pe = F2(pedge, ldp, i, nel);
        la[i - 1] = 0.0;
        if (pe == 2) {
          const double wfn = F3(sedge, 3, ldp, 1, i, nel) * n1 + F3(sedge, 3, ldp, 2, i, nel) * n2;
          const double cv = rhoA * wfn * G.meta[i - 1];
          pp = pp - cv;
        } else if (pe == 3) {
          const double ddf1 = F2(d, 2, 1, nel), ddf2 = F2(d, 2, 2, nel);
          if (intvel == 2) {
            const double dd1 = ddf1 * n1, dd2 = ddf2 * n2;
            const double ndd = dd1 * n1 + dd2 * n2;
            const double dfd = (rhoP * ndd * G.meta[i - 1]) / G.ca[i - 1];
            sp = sp + dfd;
          } else if (intvel == 5) {
            const double ndd = 0.5 * (ddf1 + ddf2);
            const double dfd = (rhoP * G.meta[i - 1] * ndd) / G.ca[i - 1];
            sp = sp + dfd;
          }
          const double wfn = F2(w, 2, 1, nel) * n1 + F2(w, 2, 2, nel) * n2;
          double cv = 0.0;
          if (fabs(wfn) > ZERO) {
            if (wfn > 0.0)
              cv = rhoP * wfn * G.meta[i - 1];
            else if (wfn < 0.0)
              cv = rhoA * wfn * G.meta[i - 1];
          }
          pp = pp - cv;
        }
      } else {
        const double alpha = G.mksif[i - 1] / G.mksi[i - 1];
        kf = (1.0 - alpha) * F2(ro, 3, 3, nel) + alpha * F2(ro, 3, 3, v);
        double ddf[2];
        ddf[0] = (1.0 - alpha) * F2(d, 2, 1, nel) + alpha * F2(d, 2, 1, v);
        ddf[1] = (1.0 - alpha) * F2(d, 2, 2, nel) + alpha * F2(d, 2, 2, v);
        double ndd;
        if (intvel == 5) {
          ndd = 0.5 * (ddf[0] + ddf[1]);
        } else {
          const double dd1 = ddf[0] * n1, dd2 = ddf[1] * n2;
          ndd = dd1 * n1 + dd2 * n2;
        }
        const double nk = n1 * G.ksi[0][i - 1] + n2 * G.ksi[1][i - 1];
        la[i - 1] = (kf * G.meta[i - 1] * ndd) / (nk * G.mksi[i - 1]);
        const double wfn = cell_vel(intvel, w, gradp, ddf, &G, p, nel, v, i, alpha);
        pp = pp - kf * wfn;
      }
    }
    if (F2(pedge, ldp, ldp, nel) == -1) sp = sp + cnst;
    la[nshared] = sp;
    for (int32_t i = 1; i <= ns; ++i) la[nshared] = la[nshared] + la[i - 1];
    double cvc;
    if (bs)
      cvc = (1.5 * F2(ro, 3, 3, nel) - 2.0 * F2(ro, 3, 2, nel) + 0.5 * F2(ro, 3, 1, nel));
    else
      cvc = (F2(ro, 3, 3, nel) - F2(ro, 3, 2, nel));
    pp = pp - G.area * cvc / dt;
    F1(rescell, nel) = fabs(pp);
    oref_assbly(ad, au, au, b, ia, ja, la, pp, ldl, nshared, matriz, unsym, 1, 1);
  }
  return 0;
}

/* EnthalpyForTemp (IdealGas.f:20-50): to_temp != 0: t = tRef + h/cP,
 * else h = cP (t - tRef); cP = e(4,1), tRef = e(5,1) (material 1). */
void oref_enthalpy_temp(double *h, double *t, const double *e, int32_t numel, int32_t to_temp) {
  const double cp = e[3], tref = e[4];
  for (int32_t i = 1; i <= numel; ++i) {
    if (to_temp)
      F1(t, i) = tref + F1(h, i) / cp;
    else
      F1(h, i) = cp * (F1(t, i) - tref);
  }
}

/* idealGas (IdealGas.f:66-91) with fIdealGas (:148-155): row `row` of
 * ro(3,*) relaxed toward P M / (R T) for air (O2/N2/Ar molar masses and
 * fractions, R, Pa and 273.15 of the reference's idealGas.fi); P = Pa
 * pressure_ratio (cPc0/cPc), celsius adds 273.15 to temp. */
void oref_ideal_gas(double *ro, const double *temp, int32_t numel, int32_t celsius, int32_t row,
                    double pressure_ratio, double under_ro) {
  const double Pa = 1.01325e5, R = 8.31431, mO2 = 32.0e-3, mN2 = 28.0e-3, mAr = 39.95e-3;
  const double dO2 = 0.21, dN2 = 0.78, dAr = 0.01, tConv = 273.15;
  const double t = celsius ? tConv : 0.0;
  const double m = dO2 * mO2 + dN2 * mN2 + dAr * mAr;
  const double P = pressure_ratio * Pa;
  for (int32_t i = 1; i <= numel; ++i) {
    const double tk = t + F1(temp, i);
    const double a = (P * m) / (R * tk);
    F2(ro, 3, row, i) = (1.0 - under_ro) * F2(ro, 3, row, i) + under_ro * a;
  }
}
