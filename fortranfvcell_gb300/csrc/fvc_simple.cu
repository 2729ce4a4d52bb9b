// fvc_simple.cu -- GPU cell kernels of the isothermal SIMPLE outer iteration
// of fortranFVCell, one thread per cell:
//   gradient   Green-Gauss over ghost / neighbour centroids (src/Pform.f:
//              466-646 gform; CellibSimple.f:895-926; CellibPressure.f:
//              577-612), momentum and pressure ghost rules
//   momentum   cell_si_eb_i_ggl iws1 = 1 (CellibSimple.f:686-894) and the
//              ideal-gas cell_si_eb_idg_ggl (CellibSimple.f:54-377): TVD
//              deferred correction, non-orthogonal correction, transposed
//              stress, second-order face pressure, under-relaxation, D, iM
//              and the cell residual; iws1 = 3 (:928-935) the time term
//   p'         cell_si_p_i_ggl iws = 1 (CellibPressure.f:477-572) with the
//              cellVel face fluxes (CellibSimple.f:1947-2073, intVel 1/2/5)
//   scatter    assbly for CSRD and ELLPACK (Assbly.f:32-54, Csr.f:142-176,
//              EllPack.f:68-93): each cell writes its own row only
//   p' (gas)   cell_si_p_idg_ggl iws = 1 (CellibPressure.f:43-246), the
//              EnthalpyForTemp and idealGas sweeps (IdealGas.f)
//   energy     cell_e_eb_idg_ggl (CellibTrans.f:39-349, ideal-gas enthalpy)
//              and cell_t_eb_ggl (CellibTrans.f:390-655, scalar transport):
//              iws 1 system, 2 gradient, 4 time term and volume source
//   sweeps     simpleUpdate, divergente (Simple.f:871-910, 1070-1078),
//              getRes (Solver.f:368-391)
// The arithmetic follows the reference statement by statement and this
// file is compiled without FMA contraction (--fmad=false), so every kernel
// reproduces the restated reference bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "fvc_internal.h"


namespace fvc {
namespace cells {
namespace {

constexpr int MS = 4;

struct Geom;
struct Mesh {
  int numel, nshared, ld;  // ld = nshared + 1 (ix rows: nodes, then material)
  const double *coor;
  const int32_t *ix, *nelcon, *num, *pedge;
  const double *sedge, *e;
  const Geom *geo;  // the cells' geometry computed once (null: per kernel)
};

__device__ __forceinline__ int ixa(const Mesh &m, int i, int c) {  // ix(i, c), 1-based
  return m.ix[(i - 1) + (size_t)(c - 1) * m.ld];
}
__device__ __forceinline__ int pedge(const Mesh &m, int i, int c) {
  return m.pedge[(i - 1) + (size_t)(c - 1) * (m.nshared + 1)];
}
__device__ __forceinline__ double sedge(const Mesh &m, int k, int i, int c) {
  return m.sedge[(k - 1) + 3 * ((size_t)(i - 1) + (size_t)(m.nshared + 1) * (c - 1))];
}
__device__ __forceinline__ double prop(const Mesh &m, int c, int i) {  // e(i, material(c))
  return m.e[(i - 1) + 10 * (size_t)(ixa(m, m.ld, c) - 1)];
}
__device__ __forceinline__ double v2(const double *a, int k, int c) {  // a(k, c), (2, *)
  return a[(k - 1) + 2 * (size_t)(c - 1)];
}

__device__ __forceinline__ double ro3(const double *ro, int k, int c) {  // ro(k, c), (3, *)
  return ro[(k - 1) + 3 * (size_t)(c - 1)];
}

struct Stencil {
  int ns;
  int viz[MS];
  int nsl[MS + 1];
  double x[2][MS][MS + 1];
};

struct Geom {
  double xc[2][MS + 1], mksi[MS], meta[MS], ksi[2][MS], n[2][MS], xm[2][MS];
  double df[2][MS], ca[MS], area;
  double xcg[2][MS], km[2][MS], mksif[MS];
};

__device__ int nsides(const Mesh &m, int c) {
  int s = 0;
  for (int i = 1; i <= m.nshared; ++i)
    if (ixa(m, i, c) > 0) ++s;
  return s;
}

__device__ void gather(Stencil &S, const Mesh &m, int nel) {
  S.ns = nsides(m, nel);
  for (int j = 1; j <= m.nshared; ++j) {
    const int v = m.nelcon[(j - 1) + (size_t)(nel - 1) * m.nshared];
    S.viz[j - 1] = v;
    if (v > 0) {
      S.nsl[j - 1] = nsides(m, v);
      for (int i = 1; i <= S.nsl[j - 1]; ++i) {
        const int no = ixa(m, i, v);
        S.x[0][i - 1][j - 1] = m.coor[2 * (size_t)(no - 1)];
        S.x[1][i - 1][j - 1] = m.coor[2 * (size_t)(no - 1) + 1];
      }
    }
  }
  S.nsl[MS] = S.ns;
  for (int i = 1; i <= S.ns; ++i) {
    const int no = ixa(m, i, nel);
    S.x[0][i - 1][MS] = m.coor[2 * (size_t)(no - 1)];
    S.x[1][i - 1][MS] = m.coor[2 * (size_t)(no - 1) + 1];
  }
}

// 0.5 |v1 x v2| with zero third components, as vet + dot_local compute it
__device__ double half_cross(double a1, double a2, double b1, double b2) {
  const double c1 = a2 * 0.0 - 0.0 * b2;
  const double c2 = 0.0 * b1 - a1 * 0.0;
  const double c3 = a1 * b2 - a2 * b1;
  const double d = ((0.0 + c1 * c1) + c2 * c2) + c3 * c3;
  return 0.5 * sqrt(d);
}

__device__ double areacell(const double eta[2][MS], int ns) {
  if (ns == 3) return half_cross(eta[0][0], eta[1][0], eta[0][1], eta[1][1]);
  double a = half_cross(eta[0][0], eta[1][0], eta[0][1], eta[1][1]);
  a = a + half_cross(eta[0][2], eta[1][2], eta[0][3], eta[1][3]);
  a = a + half_cross(eta[0][0], eta[1][0], eta[0][3], eta[1][3]);
  a = a + half_cross(eta[0][1], eta[1][1], eta[0][2], eta[1][2]);
  return 0.5 * a;
}

// the neighbour links alone (what the kernels use of the stencil when the
// geometry comes from the mesh's cache)
__device__ void gather_links(Stencil &S, const Mesh &m, int nel) {
  S.ns = nsides(m, nel);
  for (int j = 1; j <= m.nshared; ++j)
    S.viz[j - 1] = m.nelcon[(j - 1) + (size_t)(nel - 1) * m.nshared];
}

// cellGeom2D + ghost centroids + vectorKm2d for the central cell
__device__ void geom(Geom &G, const Stencil &S) {
  const int ns = S.ns;
  for (int i = 0; i < MS; ++i) {
    G.mksi[i] = 0.0;
    G.meta[i] = 0.0;
    G.ksi[0][i] = G.ksi[1][i] = 0.0;
  }
  for (int i = 1; i <= MS + 1; ++i) {
    const int slot = (i == MS + 1) ? MS : i - 1;
    if (slot < MS && (slot >= ns || S.viz[slot] <= 0)) continue;
    for (int j = 1; j <= 2; ++j) {
      double s = 0.0;
      for (int l = 1; l <= S.nsl[slot]; ++l) s = s + S.x[j - 1][l - 1][slot];
      G.xc[j - 1][slot] = (1.0 / S.nsl[slot]) * s;
    }
  }
  double eta[2][MS];
  for (int l = 1; l <= ns; ++l) {
    const int l2 = (l % ns) + 1;
    eta[0][l - 1] = S.x[0][l2 - 1][MS] - S.x[0][l - 1][MS];
    eta[1][l - 1] = S.x[1][l2 - 1][MS] - S.x[1][l - 1][MS];
  }
  G.area = areacell(eta, ns);
  for (int i = 1; i <= ns; ++i) {
    if (S.viz[i - 1] > 0) {
      for (int j = 1; j <= 2; ++j) {
        G.ksi[j - 1][i - 1] = G.xc[j - 1][i - 1] - G.xc[j - 1][MS];
        G.mksi[i - 1] = G.ksi[j - 1][i - 1] * G.ksi[j - 1][i - 1] + G.mksi[i - 1];
      }
      G.mksi[i - 1] = sqrt(G.mksi[i - 1]);
    }
  }
  for (int i = 1; i <= ns; ++i) {
    for (int j = 1; j <= 2; ++j)
      G.meta[i - 1] = G.meta[i - 1] + eta[j - 1][i - 1] * eta[j - 1][i - 1];
    G.meta[i - 1] = sqrt(G.meta[i - 1]);
  }
  for (int j = 1; j <= 2; ++j)
    for (int i = 1; i <= ns; ++i) {
      eta[j - 1][i - 1] = eta[j - 1][i - 1] / G.meta[i - 1];
      if (S.viz[i - 1] > 0) G.ksi[j - 1][i - 1] = G.ksi[j - 1][i - 1] / G.mksi[i - 1];
    }
  for (int l = 1; l <= ns; ++l) {
    G.n[0][l - 1] = eta[1][l - 1];
    G.n[1][l - 1] = -eta[0][l - 1];
  }
  for (int i = 1; i <= ns; ++i) {
    const int i2 = (i % ns) + 1;
    G.xm[0][i - 1] = 0.5 * (S.x[0][i2 - 1][MS] + S.x[0][i - 1][MS]);
    G.xm[1][i - 1] = 0.5 * (S.x[1][i2 - 1][MS] + S.x[1][i - 1][MS]);
    G.df[0][i - 1] = G.xm[0][i - 1] - G.xc[0][MS];
    G.df[1][i - 1] = G.xm[1][i - 1] - G.xc[1][MS];
    G.ca[i - 1] = G.df[0][i - 1] * G.n[0][i - 1] + G.df[1][i - 1] * G.n[1][i - 1];
  }
  for (int i = 1; i <= ns; ++i) {
    if (S.viz[i - 1] < 0) {
      for (int j = 1; j <= 2; ++j)
        G.xcg[j - 1][i - 1] = G.xc[j - 1][MS] + 2.0 * G.ca[i - 1] * G.n[j - 1][i - 1];
    } else {
      for (int j = 1; j <= 2; ++j) G.xcg[j - 1][i - 1] = G.xc[j - 1][i - 1];
    }
  }
  for (int i = 1; i <= ns; ++i) {
    const int no1 = i, no2 = (i % ns) + 1;
    const double a1 = G.xcg[1][i - 1] - G.xc[1][MS];
    const double b1 = G.xc[0][MS] - G.xcg[0][i - 1];
    const double c1 = G.xcg[0][i - 1] * G.xc[1][MS] - G.xc[0][MS] * G.xcg[1][i - 1];
    const double a2 = S.x[1][no1 - 1][MS] - S.x[1][no2 - 1][MS];
    const double b2 = S.x[0][no2 - 1][MS] - S.x[0][no1 - 1][MS];
    const double c2 =
        S.x[0][no1 - 1][MS] * S.x[1][no2 - 1][MS] - S.x[0][no2 - 1][MS] * S.x[1][no1 - 1][MS];
    const double det = a1 * b2 - a2 * b1;
    const double m11 = (1.0 / det) * b2, m12 = -(1.0 / det) * b1;
    const double m21 = -(1.0 / det) * a2, m22 = (1.0 / det) * a1;
    const double f1 = -c1, f2 = -c2;
    const double xi1 = m11 * f1 + m12 * f2, xi2 = m21 * f1 + m22 * f2;
    G.km[0][i - 1] = G.xm[0][i - 1] - xi1;
    G.km[1][i - 1] = G.xm[1][i - 1] - xi2;
    const double k1 = xi1 - G.xc[0][MS], k2 = xi2 - G.xc[1][MS];
    G.mksif[i - 1] = sqrt(k1 * k1 + k2 * k2);
  }
}

// A cell's links and geometry: from the mesh's geometry cache when it has
// one (geom() of the same stencil, stored once: the same bits), else
// computed here as the reference's cell routines do
__device__ __forceinline__ void cell_setup(Stencil &S, Geom &G, const Mesh &m, int nel) {
  if (m.geo) {
    gather_links(S, m, nel);
    G = m.geo[nel - 1];
  } else {
    gather(S, m, nel);
    geom(G, S);
  }
}

// every cell's geometry into the cache
__global__ void geometry_kernel(Mesh m, Geom *out) {
  const int nel = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (nel > m.numel) return;
  Stencil S;
  Geom G;
  gather(S, m, nel);
  geom(G, S);
  out[nel - 1] = G;
}

__device__ double limit(double r, int icod) {
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

__device__ void green_gauss(const Geom &G, int ns, const double *ug, double &g1, double &g2) {
  double eta[2][MS], n[2][MS];
  for (int i = 1; i <= 2; ++i)
    for (int l = 1; l <= ns; ++l) {
      const int s1 = l, s2 = (l % ns) + 1;
      eta[i - 1][l - 1] = G.xcg[i - 1][s2 - 1] - G.xcg[i - 1][s1 - 1];
    }
  for (int l = 1; l <= ns; ++l) {
    n[0][l - 1] = eta[1][l - 1];
    n[1][l - 1] = -eta[0][l - 1];
  }
  const double area = areacell(eta, ns);
  double um[MS];
  for (int l = 1; l <= ns; ++l) {
    const int s1 = l, s2 = (l % ns) + 1;
    um[l - 1] = 0.5 * (ug[s2 - 1] + ug[s1 - 1]);
  }
  double a = 0.0, b = 0.0;
  for (int i = 1; i <= ns; ++i) {
    const double uf = um[i - 1];
    a = a + uf * n[0][i - 1];
    b = b + uf * n[1][i - 1];
  }
  g1 = a / area;
  g2 = b / area;
}

// assbly: ld[0..nshared-1] neighbour equations (0 = none), ld[nshared] own
__device__ void assbly(double *ad, double *au, double *f, const int32_t *ia, const int32_t *ja,
                       const double *la, double p, const int *ld, int nshared, int matriz,
                       bool forces, bool matrix) {
  const int n = ld[nshared];
  if (matriz == 1) {
    if (matrix) ad[n - 1] = la[nshared];
    if (forces) f[n - 1] = p;
    const int ipont = ia[n - 1], iak = ia[n] - ia[n - 1];
    if (matrix)
      for (int j = 1; j <= nshared; ++j) {
        const int l = ld[j - 1];
        if (l > 0)
          for (int i = 1; i <= iak; ++i) {
            const int k = ipont + i - 1;
            if (l == ja[k - 1]) au[k - 1] = -la[j - 1];
          }
      }
  } else {  // 4: ELLPACK
    if (forces) f[n - 1] = p;
    if (matrix) {
      ad[n - 1] = la[nshared];
      for (int j = 1; j <= nshared; ++j) {
        const int l = ld[j - 1];
        au[(j - 1) + (size_t)(n - 1) * nshared] = (l > 0) ? -la[j - 1] : 0.0;
      }
    }
  }
}

__global__ void gradient_kernel(Mesh m, int kind, int comp, const double *__restrict__ u,
                                double *__restrict__ grad, int *err) {
  const int nel = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (nel > m.numel) return;
  Stencil S;
  Geom G;
  cell_setup(S, G, m, nel);
  const double uP = u[nel - 1];
  const double go1 = v2(grad, 1, nel), go2 = v2(grad, 2, nel);
  double ug[MS];
  for (int i = 1; i <= S.ns; ++i) {
    const int v = S.viz[i - 1];
    if (v > 0) {
      ug[i - 1] = u[v - 1];
      continue;
    }
    const int pe = pedge(m, i, nel);
    if (kind == 1) {
      if (pe == 0)
        ug[i - 1] = -uP;
      else if (pe == 1 || pe == 2)
        ug[i - 1] = sedge(m, comp, i, nel);
      else if (pe == 3 || pe == 4)
        ug[i - 1] = uP;
      else {
        atomicExch(err, 1);
        ug[i - 1] = 0.0;
      }
    } else if (kind == 3) {  // ideal-gas pressure: comp 2 = p', 3 = p
      if (pe == 3) {
        ug[i - 1] = (comp == 2) ? 0.0 : sedge(m, 3, i, nel);
      } else {
        const double gama = 2.0 * G.ca[i - 1];
        ug[i - 1] = uP + gama * (go1 * G.n[0][i - 1] + go2 * G.n[1][i - 1]);
      }
    } else {
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
  green_gauss(G, S.ns, ug, g1, g2);
  grad[2 * (size_t)(nel - 1)] = g1;
  grad[2 * (size_t)(nel - 1) + 1] = g2;
}

// idg = 1 selects the ideal-gas cell cell_si_eb_idg_ggl (CellibSimple.f:
// 54-377): densities ro(3,*) instead of e(2), the -2/3 mu div(w) terms,
// buoyancy (ro - e(2)) g A, no fixed-velocity pin
struct MomArgs {
  int comp, iws, bs, simple_c, matriz, idg;
  double dt, under_u, grav[2];
  const double *u, *u0, *w, *g_own, *g_oth, *gradp, *ro, *div;
  const int32_t *ia, *ja;
  double *ad, *au, *b, *im, *d, *rescell;
};

__global__ void momentum_kernel(Mesh m, MomArgs a) {
  const int nel = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (nel > m.numel) return;
  const double ZERO = 1.0e-7, eps = 1.0e-14, cnst = 1.0e60;
  Stencil S;
  Geom G;
  cell_setup(S, G, m, nel);
  const int ns = S.ns, nsh = m.nshared, comp = a.comp;
  const double viscosity = prop(m, nel, 1);
  const double rhoA = prop(m, nel, 2);
  const double cc = prop(m, nel, 6);
  const int icod = (int)prop(m, nel, 7);
  const double *u = a.u, *u0 = a.u0, *w = a.w, *g_own = a.g_own, *g_oth = a.g_oth;
  const double *gradp = a.gradp;
  const double uP = u[nel - 1];
  int ldl[MS + 1];
  for (int i = 0; i <= MS; ++i) ldl[i] = 0;
  for (int j = 1; j <= ns; ++j) ldl[j - 1] = (S.viz[j - 1] > 0) ? m.num[S.viz[j - 1] - 1] : 0;
  ldl[nsh] = m.num[nel - 1];
  double la[MS + 1];
  for (int i = 0; i <= MS; ++i) la[i] = 0.0;
  const bool idg = a.idg != 0;
  const double *ro = a.ro;
  if (a.iws == 3) {
    double mm = (idg ? ro3(ro, 2, nel) : prop(m, nel, 2)) * cc * G.area / a.dt;
    double p = mm * uP;
    mm = (idg ? ro3(ro, 1, nel) : prop(m, nel, 2)) * cc * G.area / a.dt;
    if (a.bs) p = 2 * p - 0.5 * mm * u0[nel - 1];
    assbly(a.ad, a.au, a.b, a.ia, a.ja, la, p, ldl, nsh, a.matriz, true, false);
    return;
  }
  const double rhoP = idg ? ro3(ro, 3, nel) : rhoA;  // the cell's current density
  double p = 0.0, pf = 0.0, sp = 0.0, cd = 0.0, cvc = 0.0;
  double aa[MS + 1];
  for (int i = 1; i <= ns; ++i) {
    const int v = S.viz[i - 1];
    const double n1 = G.n[0][i - 1], n2 = G.n[1][i - 1];
    const double meta = G.meta[i - 1];
    if (v < 0) {
      const int pe = pedge(m, i, nel);
      aa[i - 1] = 0.0;
      double ap = viscosity * meta;
      if (comp == 1)
        p = p + ap * (v2(g_own, comp, nel) * n1 + v2(g_oth, comp, nel) * n2);
      else
        p = p + ap * (v2(g_own, comp, nel) * n2 + v2(g_oth, comp, nel) * n1);
      if (idg) p = p - (2.0 / 3.0) * ap * a.div[nel - 1] * G.n[comp - 1][i - 1];
      double pface;
      if (pe == 3) {
        pface = sedge(m, 3, i, nel);
      } else {
        pface = u0[nel - 1];
        pface = pface + (v2(gradp, 1, nel) * G.df[0][i - 1] + v2(gradp, 2, nel) * G.df[1][i - 1]);
      }
      pf = pf + pface * meta * G.n[comp - 1][i - 1];
      if (pe == 0) {
        ap = viscosity * meta / G.ca[i - 1];
        sp = sp + ap;
      } else if (pe == 1) {
        ap = viscosity * meta / G.ca[i - 1];
        sp = sp + ap;
        p = p + ap * sedge(m, comp, i, nel);
      } else if (pe == 2) {
        const double wfn = sedge(m, 1, i, nel) * n1 + sedge(m, 2, i, nel) * n2;
        const double cv = rhoA * wfn * meta;
        p = p - cv * sedge(m, comp, i, nel);
      } else if (pe == 3) {
        const double wfn = v2(w, 1, nel) * n1 + v2(w, 2, nel) * n2;
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
        const double wfn = v2(w, 1, nel) * n1 + v2(w, 2, nel) * n2;
        const double cv = rhoP * wfn * meta;
        sp = sp + cv;
      }
    } else {
      double alpha = G.mksif[i - 1] / G.mksi[i - 1];
      double kf = alpha / viscosity + (1.0 - alpha) / prop(m, v, 1);
      kf = 1.0 / kf;
      const double wf1 = (1.0 - alpha) * v2(w, 1, nel) + alpha * v2(w, 1, v);
      const double wf2 = (1.0 - alpha) * v2(w, 2, nel) + alpha * v2(w, 2, v);
      double gf1 = (1.0 - alpha) * v2(g_own, 1, nel) + alpha * v2(g_own, 1, v);
      double gf2 = (1.0 - alpha) * v2(g_own, 2, nel) + alpha * v2(g_own, 2, v);
      const double k1 = G.ksi[0][i - 1], k2 = G.ksi[1][i - 1], mk = G.mksi[i - 1];
      const double nk = n1 * k1 + n2 * k2;
      const double wfn = wf1 * n1 + wf2 * n2;
      double gfk = gf1 * k1 + gf2 * k2;
      gf1 = gf1 + ((u[v - 1] - uP) / mk - gfk) * k1;
      gf2 = gf2 + ((u[v - 1] - uP) / mk - gfk) * k2;
      const double gfn = gf1 * n1 + gf2 * n2;
      gfk = gf1 * k1 + gf2 * k2;
      const double dfd = (kf * meta) / (nk * mk);
      cd = kf * meta * (gfn - gfk / nk);
      aa[i - 1] = dfd;
      p = p + cd;
      const double rof = idg ? (1.0 - alpha) * ro3(ro, 3, nel) + alpha * ro3(ro, 3, v) : rhoA;
      const double cv = rof * wfn * meta;
      if (cv < 0.0) {
        const double du = uP - u[v - 1] + eps;
        const double gpk = v2(g_own, 1, v) * (G.xc[0][MS] - G.xc[0][i - 1]) +
                           v2(g_own, 2, v) * (G.xc[1][MS] - G.xc[1][i - 1]);
        alpha = G.mksif[i - 1] / G.mksi[i - 1];
        const double r = 2.0 * gpk / du - 1.0;
        cvc = (1.0 - alpha) * limit(r, icod) * du;
      } else {
        const double du = u[v - 1] - uP + eps;
        const double gpk = (v2(g_own, 1, nel) * k1 + v2(g_own, 2, nel) * k2) * mk;
        alpha = G.mksif[i - 1] / G.mksi[i - 1];
        const double r = 2.0 * gpk / du - 1.0;
        cvc = alpha * limit(r, icod) * du;
      }
      cvc = cvc + gf1 * G.km[0][i - 1] + gf2 * G.km[1][i - 1];
      aa[i - 1] = aa[i - 1] + fmax(-cv, 0.0);
      sp = sp + cv;
      p = p - cv * cvc;
      alpha = G.mksif[i - 1] / G.mksi[i - 1];
      const double p1 = u0[nel - 1] + v2(gradp, 1, nel) * G.df[0][i - 1] +
                        v2(gradp, 2, nel) * G.df[1][i - 1];
      const double p2 = u0[v - 1] + v2(gradp, 1, v) * (G.xm[0][i - 1] - G.xc[0][i - 1]) +
                        v2(gradp, 2, v) * (G.xm[1][i - 1] - G.xc[1][i - 1]);
      const double pface = 0.5 * (p1 + p2);
      pf = pf + pface * meta * G.n[comp - 1][i - 1];
      alpha = G.mksif[i - 1] / G.mksi[i - 1];
      gf1 = (1.0 - alpha) * v2(g_own, comp, nel) + alpha * v2(g_own, comp, v);
      gf2 = (1.0 - alpha) * v2(g_oth, comp, nel) + alpha * v2(g_oth, comp, v);
      if (comp == 1)
        p = p + kf * meta * (gf1 * n1 + gf2 * n2);
      else
        p = p + kf * meta * (gf1 * n2 + gf2 * n1);
      if (idg) {  // -2/3 mu div(w) on the face
        const double gdiv = (1.0 - alpha) * a.div[nel - 1] + alpha * a.div[v - 1];
        p = p - (2.0 / 3.0) * kf * gdiv * meta * G.n[comp - 1][i - 1];
      }
    }
  }
  if (!idg && pedge(m, nsh + 1, nel) == -2) sp = sp + cnst;
  double aP = sp;
  for (int i = 1; i <= ns; ++i) aP = aP + aa[i - 1];
  double mm = rhoP * cc * G.area / a.dt;
  if (a.bs) mm = 1.5 * mm;
  aP = aP + mm;
  aP = aP / a.under_u;
  p = p + (1 - a.under_u) * aP * uP;
  if (idg)  // buoyancy (rho - rho_ref) g A with rho_ref = e(2)
    p = p + (ro3(ro, 3, nel) - rhoA) * a.grav[comp - 1] * G.area;
  double rm = 0.0, anb = 0.0;
  for (int i = 1; i <= ns; ++i) {
    rm = rm + aa[i - 1] * ((S.viz[i - 1] > 0) ? u[S.viz[i - 1] - 1] : 0.0);
    anb = anb + aa[i - 1];
  }
  a.im[(comp - 1) + 4 * (size_t)(nel - 1)] = rm + p;
  a.im[(comp + 1) + 4 * (size_t)(nel - 1)] = aP;
  if (a.simple_c)
    a.d[(comp - 1) + 2 * (size_t)(nel - 1)] = G.area / (aP - anb);
  else
    a.d[(comp - 1) + 2 * (size_t)(nel - 1)] = G.area / aP;
  p = p - pf;
  rm = p + rm - aP * uP;
  a.rescell[nel - 1] = rm;
  for (int i = 1; i <= ns; ++i) la[i - 1] = aa[i - 1];
  la[nsh] = aP;
  assbly(a.ad, a.au, a.b, a.ia, a.ja, la, p, ldl, nsh, a.matriz, true, true);
}

__device__ double cell_vel(int intvel, const double *w, const double *grad, const double ddf[2],
                           const Geom &G, const double *p, int nel, int v, int i, double alpha) {
  const double n1 = G.n[0][i - 1], n2 = G.n[1][i - 1];
  const double vm1 = (1 - alpha) * v2(w, 1, nel) + alpha * v2(w, 1, v);
  const double vm2 = (1 - alpha) * v2(w, 2, nel) + alpha * v2(w, 2, v);
  double wfn = vm1 * n1 + vm2 * n2;
  if (intvel == 1) return wfn * G.meta[i - 1];
  const double gf1 = (1 - alpha) * v2(grad, 1, nel) + alpha * v2(grad, 1, v);
  const double gf2 = (1 - alpha) * v2(grad, 2, nel) + alpha * v2(grad, 2, v);
  if (intvel == 2) {
    const double gfp1 = ((p[v - 1] - p[nel - 1]) / G.mksi[i - 1]);
    const double gfp2 = gf1 * G.ksi[0][i - 1] + gf2 * G.ksi[1][i - 1];
    wfn = wfn + 0.5 * (ddf[0] + ddf[1]) * (gfp2 - gfp1);
    return wfn * G.meta[i - 1];
  }
  const double gfp1 = p[v - 1] - p[nel - 1];
  const double ks1 = G.mksi[i - 1] * G.ksi[0][i - 1];
  const double ks2 = G.mksi[i - 1] * G.ksi[1][i - 1];
  const double nk = ks1 * n1 + ks2 * n2;
  double gfp2 = gf1 * ks1 + gf2 * ks2;
  gfp2 = (gfp2 - gfp1) / nk;
  wfn = wfn + 0.5 * (ddf[0] + ddf[1]) * gfp2;
  return wfn * G.meta[i - 1];
}

struct PcArgs {
  int intvel, matriz;
  const double *w, *d, *p, *gradp;
  const int32_t *ia, *ja;
  double *ad, *au, *b, *rescell;
};

__global__ void pc_kernel(Mesh m, PcArgs a) {
  const int nel = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (nel > m.numel) return;
  const double cnst = 1.0e60;
  Stencil S;
  Geom G;
  cell_setup(S, G, m, nel);
  const int ns = S.ns, nsh = m.nshared;
  const double rhoA = prop(m, nel, 2);
  const double *w = a.w, *d = a.d;
  int ldl[MS + 1];
  for (int i = 0; i <= MS; ++i) ldl[i] = 0;
  for (int j = 1; j <= ns; ++j) ldl[j - 1] = (S.viz[j - 1] > 0) ? m.num[S.viz[j - 1] - 1] : 0;
  ldl[nsh] = m.num[nel - 1];
  double la[MS + 1];
  for (int i = 0; i <= MS; ++i) la[i] = 0.0;
  double pp = 0.0, sp = 0.0, kf = 0.0;
  for (int i = 1; i <= ns; ++i) {
    const int v = S.viz[i - 1];
    const double n1 = G.n[0][i - 1], n2 = G.n[1][i - 1];
    if (v < 0) {
      const int pe = pedge(m, i, nel);
      la[i - 1] = 0.0;
      if (pe == 2 || pe == 4) {
        const double wfn = sedge(m, 1, i, nel) * n1 + sedge(m, 2, i, nel) * n2;
        const double cv = rhoA * wfn * G.meta[i - 1];
        pp = pp - cv;
      } else if (pe == 3) {
        const double dd1 = v2(d, 1, nel) * n1, dd2 = v2(d, 2, nel) * n2;
        const double ndd = dd1 * n1 + dd2 * n2;
        const double dfd = (rhoA * ndd * G.meta[i - 1]) / G.ca[i - 1];
        sp = sp + dfd;
        const double wfn = v2(w, 1, nel) * n1 + v2(w, 2, nel) * n2;
        const double cv = rhoA * wfn * G.meta[i - 1];
        pp = pp - cv;
      }
    } else {
      const double alpha = G.mksif[i - 1] / G.mksi[i - 1];
      double ddf[2], ndd;
      if (a.intvel == 5) {
        kf = (1.0 - alpha) * prop(m, nel, 2) + alpha * prop(m, v, 2);
        ddf[0] = (1.0 - alpha) * v2(d, 1, nel) + alpha * v2(d, 1, v);
        ddf[1] = (1.0 - alpha) * v2(d, 2, nel) + alpha * v2(d, 2, v);
        ndd = 0.5 * (ddf[0] + ddf[1]);
      } else {
        kf = prop(m, nel, 2);
        ddf[0] = (1.0 - alpha) * v2(d, 1, nel) + alpha * v2(d, 1, v);
        ddf[1] = (1.0 - alpha) * v2(d, 2, nel) + alpha * v2(d, 2, v);
        const double dd1 = ddf[0] * n1, dd2 = ddf[1] * n2;
        ndd = dd1 * n1 + dd2 * n2;
      }
      const double nk = n1 * G.ksi[0][i - 1] + n2 * G.ksi[1][i - 1];
      la[i - 1] = (kf * G.meta[i - 1] * ndd) / (nk * G.mksi[i - 1]);
      const double wfn = cell_vel(a.intvel, w, a.gradp, ddf, G, a.p, nel, v, i, alpha);
      pp = pp - kf * wfn;
    }
  }
  if (pedge(m, nsh + 1, nel) == -1) sp = sp + cnst;
  la[nsh] = sp;
  for (int i = 1; i <= ns; ++i) la[nsh] = la[nsh] + la[i - 1];
  a.rescell[nel - 1] = pp;
  assbly(a.ad, a.au, a.b, a.ia, a.ja, la, pp, ldl, nsh, a.matriz, true, true);
}

__global__ void simple_update_kernel(int numel, double *w, double *pre, const double *u1,
                                     const double *u2, const double *prec, const double *gpc,
                                     const double *d, double under_pc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= numel) return;
  w[2 * (size_t)i] = u1[i] - d[2 * (size_t)i] * gpc[2 * (size_t)i];
  w[2 * (size_t)i + 1] = u2[i] - d[2 * (size_t)i + 1] * gpc[2 * (size_t)i + 1];
  pre[i] = pre[i] + under_pc * prec[i];
}

__global__ void divergence_kernel(int numel, double *div, const double *gu1, const double *gu2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < numel) div[i] = gu1[2 * (size_t)i] + gu2[2 * (size_t)i + 1];
}

__global__ void getres_kernel(int numel, const int32_t *num, double *u, double *x, int to_eq) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= numel) return;
  if (to_eq)
    x[num[i] - 1] = u[i];
  else
    u[i] = x[num[i] - 1];
}

// ---- ideal gas: p' cell (CellibPressure.f:43-246), property sweeps --------
struct PcIdgArgs {
  int intvel, matriz, bs;
  double dt;
  const double *w, *d, *p, *gradp, *ro;
  const int32_t *ia, *ja;
  double *ad, *au, *b, *rescell;
};

__global__ void pc_idg_kernel(Mesh m, PcIdgArgs a) {
  const int nel = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (nel > m.numel) return;
  const double cnst = 1.0e60, ZERO = 1.0e-7;
  Stencil S;
  Geom G;
  cell_setup(S, G, m, nel);
  const int ns = S.ns, nsh = m.nshared;
  const double *w = a.w, *d = a.d, *ro = a.ro;
  const double rhoP = ro3(ro, 3, nel), rhoA = prop(m, nel, 2);
  int ldl[MS + 1];
  for (int i = 0; i <= MS; ++i) ldl[i] = 0;
  for (int j = 1; j <= ns; ++j) ldl[j - 1] = (S.viz[j - 1] > 0) ? m.num[S.viz[j - 1] - 1] : 0;
  ldl[nsh] = m.num[nel - 1];
  double la[MS + 1];
  for (int i = 0; i <= MS; ++i) la[i] = 0.0;
  double pp = 0.0, sp = 0.0, kf = 0.0;
  for (int i = 1; i <= ns; ++i) {
    const int v = S.viz[i - 1];
    const double n1 = G.n[0][i - 1], n2 = G.n[1][i - 1];
    if (v < 0) {
      const int pe = pedge(m, i, nel);
      la[i - 1] = 0.0;
      if (pe == 2) {
        const double wfn = sedge(m, 1, i, nel) * n1 + sedge(m, 2, i, nel) * n2;
        const double cv = rhoA * wfn * G.meta[i - 1];
        pp = pp - cv;
      } else if (pe == 3) {
        const double ddf1 = v2(d, 1, nel), ddf2 = v2(d, 2, nel);
        if (a.intvel == 2) {
          const double dd1 = ddf1 * n1, dd2 = ddf2 * n2;
          const double ndd = dd1 * n1 + dd2 * n2;
          const double dfd = (rhoP * ndd * G.meta[i - 1]) / G.ca[i - 1];
          sp = sp + dfd;
        } else if (a.intvel == 5) {
          const double ndd = 0.5 * (ddf1 + ddf2);
          const double dfd = (rhoP * G.meta[i - 1] * ndd) / G.ca[i - 1];
          sp = sp + dfd;
        }
        const double wfn = v2(w, 1, nel) * n1 + v2(w, 2, nel) * n2;
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
      kf = (1.0 - alpha) * ro3(ro, 3, nel) + alpha * ro3(ro, 3, v);
      double ddf[2];
      ddf[0] = (1.0 - alpha) * v2(d, 1, nel) + alpha * v2(d, 1, v);
      ddf[1] = (1.0 - alpha) * v2(d, 2, nel) + alpha * v2(d, 2, v);
      double ndd;
      if (a.intvel == 5) {
        ndd = 0.5 * (ddf[0] + ddf[1]);
      } else {
        const double dd1 = ddf[0] * n1, dd2 = ddf[1] * n2;
        ndd = dd1 * n1 + dd2 * n2;
      }
      const double nk = n1 * G.ksi[0][i - 1] + n2 * G.ksi[1][i - 1];
      la[i - 1] = (kf * G.meta[i - 1] * ndd) / (nk * G.mksi[i - 1]);
      const double wfn = cell_vel(a.intvel, w, a.gradp, ddf, G, a.p, nel, v, i, alpha);
      pp = pp - kf * wfn;
    }
  }
  if (pedge(m, nsh + 1, nel) == -1) sp = sp + cnst;
  la[nsh] = sp;
  for (int i = 1; i <= ns; ++i) la[nsh] = la[nsh] + la[i - 1];
  double cvc;
  if (a.bs)
    cvc = (1.5 * ro3(ro, 3, nel) - 2.0 * ro3(ro, 2, nel) + 0.5 * ro3(ro, 1, nel));
  else
    cvc = (ro3(ro, 3, nel) - ro3(ro, 2, nel));
  pp = pp - G.area * cvc / a.dt;
  a.rescell[nel - 1] = fabs(pp);
  assbly(a.ad, a.au, a.b, a.ia, a.ja, la, pp, ldl, nsh, a.matriz, true, true);
}

// EnthalpyForTemp (IdealGas.f:20-50): to_temp: t = tRef + h/cP, else
// h = cP (t - tRef)
__global__ void enthalpy_temp_kernel(int numel, double *h, double *t, double cp, double tref,
                                     int to_temp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= numel) return;
  if (to_temp)
    t[i] = tref + h[i] / cp;
  else
    h[i] = cp * (t[i] - tref);
}

// idealGas with fIdealGas (IdealGas.f:66-91,148-155): air of the reference's
// idealGas.fi (O2/N2/Ar molar masses and fractions, R, Pa, 273.15)
__global__ void ideal_gas_kernel(int numel, double *ro, const double *temp, int celsius, int row,
                                 double pressure_ratio, double under_ro) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= numel) return;
  const double Pa = 1.01325e5, R = 8.31431, mO2 = 32.0e-3, mN2 = 28.0e-3, mAr = 39.95e-3;
  const double dO2 = 0.21, dN2 = 0.78, dAr = 0.01, tConv = 273.15;
  const double t = celsius ? tConv : 0.0;
  const double mm = dO2 * mO2 + dN2 * mN2 + dAr * mAr;
  const double P = pressure_ratio * Pa;
  const double tk = t + temp[i];
  const double av = (P * mm) / (R * tk);
  double &r = ro[(row - 1) + 3 * (size_t)i];
  r = (1.0 - under_ro) * r + under_ro * av;
}

// ---- energy / scalar transport cells (src/CellibTrans.f) -----------------
// lib 3: cell_e_eb_idg_ggl (ideal-gas enthalpy, CellibTrans.f:39-349);
// lib 4: cell_t_eb_ggl (scalar transport, CellibTrans.f:390-655).  The
// scalar's own boundary arrays pe(nshared+1,*), se(nshared+1,*) (one value
// per face; face nshared+1 a volume source).  ro(3,*): densities at n-1, n
// and the current iterate.  The reference declares the boundary enthalpy
// of lib 3 and the inflow density of lib 4 integer: both are truncated
// toward zero here as there.
struct EnArgs {
  int lib, iws, bs, matriz;
  double dt;
  const int32_t *pe;
  const double *se;
  const double *u, *u0, *ro, *w, *grad;
  const int32_t *ia, *ja;
  double *ad, *au, *b, *rescell;
};

__device__ __forceinline__ int epedge(const int32_t *pe, int nsh, int i, int c) {
  return pe[(i - 1) + (size_t)(c - 1) * (nsh + 1)];
}
__device__ __forceinline__ double esedge(const double *se, int nsh, int i, int c) {
  return se[(i - 1) + (size_t)(c - 1) * (nsh + 1)];
}

__global__ void energy_gradient_kernel(Mesh m, int lib, const int32_t *__restrict__ pe,
                                       const double *__restrict__ se,
                                       const double *__restrict__ u, double *__restrict__ grad) {
  const int nel = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (nel > m.numel) return;
  Stencil S;
  Geom G;
  cell_setup(S, G, m, nel);
  const double uP = u[nel - 1];
  const double go1 = v2(grad, 1, nel), go2 = v2(grad, 2, nel);
  const double cesp = prop(m, nel, 4), tref = prop(m, nel, 5);
  double ug[MS];
  for (int i = 1; i <= S.ns; ++i) {
    const int v = S.viz[i - 1];
    if (v > 0) {
      ug[i - 1] = u[v - 1];
      continue;
    }
    const int pcode = epedge(pe, m.nshared, i, nel);
    const double sface = esedge(se, m.nshared, i, nel);
    if (lib == 3) {  // CellibTrans.f:131-144
      if (pcode == 2) {
        const int enthalpia = (int)(cesp * (sface - tref));
        ug[i - 1] = (double)enthalpia;
      } else {
        const double gama = 2.0 * G.ca[i - 1];
        ug[i - 1] = uP + gama * (go1 * G.n[0][i - 1] + go2 * G.n[1][i - 1]);
      }
    } else {  // CellibTrans.f:460-464
      ug[i - 1] = (pcode == 2) ? 2.0 * sface - uP : uP;
    }
  }
  double g1, g2;
  green_gauss(G, S.ns, ug, g1, g2);
  grad[2 * (size_t)(nel - 1)] = g1;
  grad[2 * (size_t)(nel - 1) + 1] = g2;
}

__global__ void energy_kernel(Mesh m, EnArgs a) {
  const int nel = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (nel > m.numel) return;
  const double ZERO = 1.0e-14, eps = 1.0e-14;
  Stencil S;
  Geom G;
  cell_setup(S, G, m, nel);
  const int ns = S.ns, nsh = m.nshared, lib = a.lib;
  const double kc = prop(m, nel, 3);
  const double cesp = prop(m, nel, 4);
  const double tref = prop(m, nel, 5);
  const double cc = prop(m, nel, 6);
  const int icod = (int)prop(m, nel, 7);
  const int spec_mass = (int)prop(m, nel, 2);  // lib 4: an integer in the reference
  const double *u = a.u, *ro = a.ro, *w = a.w, *grad = a.grad;
  const double uP = u[nel - 1];
  int ldl[MS + 1];
  for (int i = 0; i <= MS; ++i) ldl[i] = 0;
  for (int j = 1; j <= ns; ++j) ldl[j - 1] = (S.viz[j - 1] > 0) ? m.num[S.viz[j - 1] - 1] : 0;
  ldl[nsh] = m.num[nel - 1];
  double la[MS + 1];
  for (int i = 0; i <= MS; ++i) la[i] = 0.0;
  if (a.iws == 4) {  // label 400: time term and volume source
    double mm = ro3(ro, 2, nel) * cc * G.area / a.dt;
    double p = mm * uP;
    if (a.bs) {
      mm = ro3(ro, 1, nel) * cc * G.area / a.dt;
      p = 2 * p - 0.5 * mm * a.u0[nel - 1];
    }
    if (epedge(a.pe, nsh, nsh + 1, nel) != 0) p = p + esedge(a.se, nsh, nsh + 1, nel) * G.area;
    assbly(a.ad, a.au, a.b, a.ia, a.ja, la, p, ldl, nsh, a.matriz, true, false);
    return;
  }
  const double roc = ro3(ro, 3, nel);
  double rof = roc;  // lib 4 carries it from face to face
  double p = 0.0, sp = 0.0, cd = 0.0, cvc = 0.0;
  double aa[MS];
  for (int i = 1; i <= ns; ++i) {
    const int v = S.viz[i - 1];
    const double n1 = G.n[0][i - 1], n2 = G.n[1][i - 1];
    const double meta = G.meta[i - 1];
    if (v < 0) {
      const int pcode = epedge(a.pe, nsh, i, nel);
      const double sface = esedge(a.se, nsh, i, nel);
      aa[i - 1] = 0.0;
      const double wfn = v2(w, 1, nel) * n1 + v2(w, 2, nel) * n2;
      double cv = (lib == 3 ? roc : rof) * wfn * meta;
      if (pcode == 0) {
        p = p + sface * meta;
      } else if (pcode == 1) {
        if (lib == 3) {
          const double ap = (kc / cesp) * meta / G.ca[i - 1];
          sp = sp + ap;
          const int enthalpia = (int)(cesp * (sface - tref));
          p = p + ap * enthalpia;
        } else {
          const double ap = kc * meta / G.ca[i - 1];
          sp = sp + ap;
          p = p + ap * sface;
        }
      } else if (pcode == 2) {
        if (lib == 3) {
          if (fabs(wfn) > ZERO) {
            if (cv < 0.0) {
              cv = prop(m, nel, 2) * wfn * meta;
              const int enthalpia = (int)(cesp * (sface - tref));
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
      } else if (pcode == 4) {
        sp = sp + cv;
      }
    } else {
      double alpha = G.mksif[i - 1] / G.mksi[i - 1];
      double kf;
      if (lib == 3)
        kf = alpha / (kc / cesp) + (1.0 - alpha) / (prop(m, v, 3) / prop(m, v, 4));
      else
        kf = alpha / kc + (1.0 - alpha) / prop(m, v, 3);
      kf = 1.0 / kf;
      const double wf1 = (1.0 - alpha) * v2(w, 1, nel) + alpha * v2(w, 1, v);
      const double wf2 = (1.0 - alpha) * v2(w, 2, nel) + alpha * v2(w, 2, v);
      double gf1 = (1.0 - alpha) * v2(grad, 1, nel) + alpha * v2(grad, 1, v);
      double gf2 = (1.0 - alpha) * v2(grad, 2, nel) + alpha * v2(grad, 2, v);
      const double k1 = G.ksi[0][i - 1], k2 = G.ksi[1][i - 1], mk = G.mksi[i - 1];
      const double nk = n1 * k1 + n2 * k2;
      const double wfn = wf1 * n1 + wf2 * n2;
      const double uv = u[v - 1];
      double gfk = gf1 * k1 + gf2 * k2;
      gf1 = gf1 + ((uv - uP) / mk - gfk) * k1;
      gf2 = gf2 + ((uv - uP) / mk - gfk) * k2;
      const double gfn = gf1 * n1 + gf2 * n2;
      gfk = gf1 * k1 + gf2 * k2;
      const double dfd = (kf * meta) / (nk * mk);
      cd = kf * meta * (gfn - gfk / nk);
      aa[i - 1] = dfd;
      p = p + cd;
      if (lib == 3) {
        rof = (1.0 - alpha) * ro3(ro, 3, nel) + alpha * ro3(ro, 3, v);
      } else {
        if (wfn > 0.0)
          rof = ro3(ro, 3, nel);
        else if (wfn < 0.0)
          rof = ro3(ro, 3, v);
        else
          rof = (1.0 - alpha) * ro3(ro, 3, nel) + alpha * ro3(ro, 3, v);
      }
      const double cv = rof * wfn * meta;
      if (cv < 0.0) {
        const double du = uP - uv + eps;
        const double gpk = v2(grad, 1, v) * (G.xc[0][MS] - G.xc[0][i - 1]) +
                           v2(grad, 2, v) * (G.xc[1][MS] - G.xc[1][i - 1]);
        alpha = G.mksif[i - 1] / G.mksi[i - 1];
        const double r = 2.0 * gpk / du - 1.0;
        cvc = (1.0 - alpha) * limit(r, icod) * du;
      } else {
        const double du = uv - uP + eps;
        const double gpk = (v2(grad, 1, nel) * k1 + v2(grad, 2, nel) * k2) * mk;
        alpha = G.mksif[i - 1] / G.mksi[i - 1];
        const double r = 2.0 * gpk / du - 1.0;
        cvc = alpha * limit(r, icod) * du;
      }
      cvc = cvc + gf1 * G.km[0][i - 1] + gf2 * G.km[1][i - 1];
      aa[i - 1] = aa[i - 1] + fmax(-cv, 0.0);
      sp = sp + cv;
      p = p - cv * cvc;
    }
  }
  double aP = sp;
  for (int i = 1; i <= ns; ++i) aP = aP + aa[i - 1];
  double mm = ro3(ro, 3, nel) * cc * G.area / a.dt;
  if (a.bs) mm = 1.5 * mm;
  aP = aP + mm;
  double rm = p - aP * uP;
  for (int i = 1; i <= ns; ++i)
    rm = rm + aa[i - 1] * ((S.viz[i - 1] > 0) ? u[S.viz[i - 1] - 1] : 0.0);
  a.rescell[nel - 1] = rm;
  for (int i = 1; i <= ns; ++i) la[i - 1] = aa[i - 1];
  la[nsh] = aP;
  assbly(a.ad, a.au, a.b, a.ia, a.ja, la, p, ldl, nsh, a.matriz, true, true);
}

Mesh view(const fvc_cell_mesh *m) {
  Mesh v;
  v.numel = m->numel;
  v.nshared = m->nshared;
  v.ld = m->nshared + 1;
  v.coor = m->coor;
  v.ix = m->ix;
  v.nelcon = m->nelcon;
  v.num = m->num;
  v.pedge = m->pedge;
  v.sedge = m->sedge;
  v.e = m->e;
  v.geo = static_cast<const Geom *>(m->geometry);
  return v;
}

bool mesh_ok(const fvc_cell_mesh *m) {
  return m && m->numel > 0 && (m->nshared == 3 || m->nshared == 4) && m->coor && m->ix &&
         m->nelcon && m->num && m->pedge && m->sedge && m->e;
}

// the energy cells take their own boundary arrays: geometry and materials only
bool mesh_geom_ok(const fvc_cell_mesh *m) {
  return m && m->numel > 0 && (m->nshared == 3 || m->nshared == 4) && m->coor && m->ix &&
         m->nelcon && m->num && m->e;
}

constexpr int kThreads = 128;
inline int grid(int n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

int32_t gradient_async(const fvc_cell_mesh *m, int kind, int comp, const double *u,
                       double *grad, int *d_err, cudaStream_t s) {
  if (!mesh_ok(m) || !u || !grad || !d_err || kind < 1 || kind > 3 || comp < 1 || comp > 3 ||
      (kind == 3 && comp == 1))
    return FVC_ERR_ARG;
  gradient_kernel<<<grid(m->numel), kThreads, 0, s>>>(view(m), kind, comp, u, grad, d_err);
  count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t gradient(const fvc_cell_mesh *m, int kind, int comp, const double *u, double *grad,
                 cudaStream_t s) {
  if (!mesh_ok(m) || !u || !grad || kind < 1 || kind > 3 || comp < 1 || comp > 3 ||
      (kind == 3 && comp == 1))
    return FVC_ERR_ARG;
  int *err = nullptr;
  if (cudaMallocAsync(&err, sizeof(int), s) != cudaSuccess) return FVC_ERR_CUDA;
  cudaMemsetAsync(err, 0, sizeof(int), s);
  gradient_kernel<<<grid(m->numel), kThreads, 0, s>>>(view(m), kind, comp, u, grad, err);
  count_launch();
  int herr = 0;
  cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(err, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return FVC_ERR_CUDA;
  return herr ? FVC_ERR_UNSUPPORTED : FVC_OK;
}

}  // namespace cells
}  // namespace fvc

using fvc::cells::grid;
using fvc::cells::kThreads;

extern "C" {

int32_t fvc_cells_gradient(const fvc_cell_mesh *m, int32_t kind, int32_t comp, const double *u,
                           double *grad, void *stream) {
  return fvc::cells::gradient(m, kind, comp, u, grad, (cudaStream_t)stream);
}

int32_t fvc_cells_momentum(const fvc_cell_mesh *m, int32_t comp, int32_t iws, const double *u,
                           const double *u0, const double *w, const double *g_own,
                           const double *g_oth, const double *gradp, double dt, int32_t bs,
                           double under_u, int32_t simple_c, int32_t matriz, const int32_t *ia,
                           const int32_t *ja, double *ad, double *au, double *b, double *im,
                           double *d, double *rescell, void *stream) {
  if (!fvc::cells::mesh_ok(m) || (comp != 1 && comp != 2) || (iws != 1 && iws != 3) ||
      (matriz != 1 && matriz != 4) || !u || !b || dt == 0.0)
    return FVC_ERR_ARG;
  if (iws == 1 && (!w || !g_own || !g_oth || !gradp || !ad || !au || !im || !d || !rescell ||
                   !u0 || (matriz == 1 && (!ia || !ja))))
    return FVC_ERR_ARG;
  if (iws == 3 && bs && !u0) return FVC_ERR_ARG;
  fvc::cells::MomArgs a;
  a.comp = comp;
  a.iws = iws;
  a.bs = bs;
  a.simple_c = simple_c;
  a.matriz = matriz;
  a.dt = dt;
  a.under_u = under_u;
  a.u = u;
  a.u0 = u0;
  a.w = w;
  a.g_own = g_own;
  a.g_oth = g_oth;
  a.gradp = gradp;
  a.ia = ia;
  a.ja = ja;
  a.ad = ad;
  a.au = au;
  a.b = b;
  a.im = im;
  a.d = d;
  a.rescell = rescell;
  a.idg = 0;
  a.ro = nullptr;
  a.div = nullptr;
  a.grav[0] = a.grav[1] = 0.0;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::momentum_kernel<<<grid(m->numel), kThreads, 0, s>>>(fvc::cells::view(m), a);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_cells_momentum_ideal_gas(const fvc_cell_mesh *m, int32_t comp, int32_t iws,
                                     const double *u, const double *u0, const double *w,
                                     const double *g_own, const double *g_oth,
                                     const double *gradp, const double *ro, const double *div,
                                     double gx, double gy, double dt, int32_t bs, double under_u,
                                     int32_t simple_c, int32_t matriz, const int32_t *ia,
                                     const int32_t *ja, double *ad, double *au, double *b,
                                     double *im, double *d, double *rescell, void *stream) {
  if (!fvc::cells::mesh_ok(m) || (comp != 1 && comp != 2) || (iws != 1 && iws != 3) ||
      (matriz != 1 && matriz != 4) || !u || !b || !ro || dt == 0.0)
    return FVC_ERR_ARG;
  if (iws == 1 && (!w || !g_own || !g_oth || !gradp || !div || !ad || !au || !im || !d ||
                   !rescell || !u0 || (matriz == 1 && (!ia || !ja))))
    return FVC_ERR_ARG;
  if (iws == 3 && bs && !u0) return FVC_ERR_ARG;
  fvc::cells::MomArgs a;
  a.comp = comp;
  a.iws = iws;
  a.bs = bs;
  a.simple_c = simple_c;
  a.matriz = matriz;
  a.idg = 1;
  a.dt = dt;
  a.under_u = under_u;
  a.grav[0] = gx;
  a.grav[1] = gy;
  a.u = u;
  a.u0 = u0;
  a.w = w;
  a.g_own = g_own;
  a.g_oth = g_oth;
  a.gradp = gradp;
  a.ro = ro;
  a.div = div;
  a.ia = ia;
  a.ja = ja;
  a.ad = ad;
  a.au = au;
  a.b = b;
  a.im = im;
  a.d = d;
  a.rescell = rescell;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::momentum_kernel<<<grid(m->numel), kThreads, 0, s>>>(fvc::cells::view(m), a);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_cells_pressure_correction(const fvc_cell_mesh *m, const double *w, const double *d,
                                      const double *p, const double *gradp, int32_t int_vel,
                                      int32_t matriz, const int32_t *ia, const int32_t *ja,
                                      double *ad, double *au, double *b, double *rescell,
                                      void *stream) {
  if (!fvc::cells::mesh_ok(m) || !w || !d || !p || !gradp || !ad || !au || !b || !rescell ||
      (matriz != 1 && matriz != 4) || (matriz == 1 && (!ia || !ja)))
    return FVC_ERR_ARG;
  // cellVel leaves the face flux undefined for intVel 3, 4 and 6
  if (int_vel != 1 && int_vel != 2 && int_vel != 5) return FVC_ERR_UNSUPPORTED;
  fvc::cells::PcArgs a;
  a.intvel = int_vel;
  a.matriz = matriz;
  a.w = w;
  a.d = d;
  a.p = p;
  a.gradp = gradp;
  a.ia = ia;
  a.ja = ja;
  a.ad = ad;
  a.au = au;
  a.b = b;
  a.rescell = rescell;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::pc_kernel<<<grid(m->numel), kThreads, 0, s>>>(fvc::cells::view(m), a);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_cells_pressure_correction_ideal_gas(const fvc_cell_mesh *m, const double *w,
                                                const double *d, const double *p,
                                                const double *gradp, const double *ro,
                                                int32_t int_vel, double dt, int32_t bs,
                                                int32_t matriz, const int32_t *ia,
                                                const int32_t *ja, double *ad, double *au,
                                                double *b, double *rescell, void *stream) {
  if (!fvc::cells::mesh_ok(m) || !w || !d || !p || !gradp || !ro || !ad || !au || !b ||
      !rescell || (matriz != 1 && matriz != 4) || (matriz == 1 && (!ia || !ja)) || dt == 0.0)
    return FVC_ERR_ARG;
  if (int_vel != 1 && int_vel != 2 && int_vel != 5) return FVC_ERR_UNSUPPORTED;
  fvc::cells::PcIdgArgs a;
  a.intvel = int_vel;
  a.matriz = matriz;
  a.bs = bs;
  a.dt = dt;
  a.w = w;
  a.d = d;
  a.p = p;
  a.gradp = gradp;
  a.ro = ro;
  a.ia = ia;
  a.ja = ja;
  a.ad = ad;
  a.au = au;
  a.b = b;
  a.rescell = rescell;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::pc_idg_kernel<<<grid(m->numel), kThreads, 0, s>>>(fvc::cells::view(m), a);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_cells_enthalpy_temperature(int32_t numel, double *h, double *t, double cp,
                                       double tref, int32_t to_temperature, void *stream) {
  if (numel <= 0 || !h || !t || cp == 0.0) return FVC_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::enthalpy_temp_kernel<<<grid(numel), kThreads, 0, s>>>(numel, h, t, cp, tref,
                                                                    to_temperature ? 1 : 0);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_cells_ideal_gas_density(int32_t numel, double *ro, const double *temp,
                                    int32_t celsius, int32_t row, double pressure_ratio,
                                    double under_ro, void *stream) {
  if (numel <= 0 || !ro || !temp || row < 1 || row > 3) return FVC_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::ideal_gas_kernel<<<grid(numel), kThreads, 0, s>>>(
      numel, ro, temp, celsius ? 1 : 0, row, pressure_ratio, under_ro);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_cells_simple_update(int32_t numel, double *w, double *p, const double *u1,
                                const double *u2, const double *pc, const double *gradpc,
                                const double *d, double under_pc, void *stream) {
  if (numel <= 0 || !w || !p || !u1 || !u2 || !pc || !gradpc || !d) return FVC_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::simple_update_kernel<<<grid(numel), kThreads, 0, s>>>(numel, w, p, u1, u2, pc,
                                                                    gradpc, d, under_pc);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_cells_divergence(int32_t numel, double *div, const double *gu1, const double *gu2,
                             void *stream) {
  if (numel <= 0 || !div || !gu1 || !gu2) return FVC_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::divergence_kernel<<<grid(numel), kThreads, 0, s>>>(numel, div, gu1, gu2);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_cells_energy_gradient(const fvc_cell_mesh *m, int32_t lib, const int32_t *pedge,
                                  const double *sedge, const double *u, double *grad,
                                  void *stream) {
  if (!fvc::cells::mesh_geom_ok(m) || (lib != 3 && lib != 4) || !pedge || !sedge || !u || !grad)
    return FVC_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::energy_gradient_kernel<<<grid(m->numel), kThreads, 0, s>>>(
      fvc::cells::view(m), lib, pedge, sedge, u, grad);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_cells_energy(const fvc_cell_mesh *m, int32_t lib, int32_t iws, const int32_t *pedge,
                         const double *sedge, const double *u, const double *u0,
                         const double *ro, const double *w, const double *grad, double dt,
                         int32_t bs, int32_t matriz, const int32_t *ia, const int32_t *ja,
                         double *ad, double *au, double *b, double *rescell, void *stream) {
  if (!fvc::cells::mesh_geom_ok(m) || (lib != 3 && lib != 4) || (iws != 1 && iws != 4) ||
      (matriz != 1 && matriz != 4) || !pedge || !sedge || !u || !ro || !b || dt == 0.0)
    return FVC_ERR_ARG;
  if (iws == 1 && (!w || !grad || !ad || !au || !rescell || (matriz == 1 && (!ia || !ja))))
    return FVC_ERR_ARG;
  if (iws == 4 && bs && !u0) return FVC_ERR_ARG;
  fvc::cells::EnArgs a;
  a.lib = lib;
  a.iws = iws;
  a.bs = bs;
  a.matriz = matriz;
  a.dt = dt;
  a.pe = pedge;
  a.se = sedge;
  a.u = u;
  a.u0 = u0;
  a.ro = ro;
  a.w = w;
  a.grad = grad;
  a.ia = ia;
  a.ja = ja;
  a.ad = ad;
  a.au = au;
  a.b = b;
  a.rescell = rescell;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::energy_kernel<<<grid(m->numel), kThreads, 0, s>>>(fvc::cells::view(m), a);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_getres(int32_t numel, const int32_t *num, double *u, double *x, int32_t to_equations,
                   void *stream) {
  if (numel <= 0 || !num || !u || !x) return FVC_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  fvc::cells::getres_kernel<<<grid(numel), kThreads, 0, s>>>(numel, num, u, x,
                                                              to_equations ? 1 : 0);
  fvc::count_launch();
  return cudaPeekAtLastError() == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}

int32_t fvc_cells_geometry_create(const fvc_cell_mesh *m, void **geometry) {
  if (!geometry || !m || m->numel <= 0 || (m->nshared != 3 && m->nshared != 4) || !m->coor ||
      !m->ix || !m->nelcon)
    return FVC_ERR_ARG;
  *geometry = nullptr;
  fvc::cells::Geom *g = nullptr;
  if (cudaMalloc(&g, sizeof(fvc::cells::Geom) * (size_t)m->numel) != cudaSuccess)
    return FVC_ERR_CUDA;
  fvc::cells::Mesh v = fvc::cells::view(m);
  v.geo = nullptr;
  fvc::cells::geometry_kernel<<<fvc::cells::grid(m->numel), fvc::cells::kThreads>>>(v, g);
  fvc::count_launch();
  if (cudaDeviceSynchronize() != cudaSuccess) {
    cudaFree(g);
    return FVC_ERR_CUDA;
  }
  *geometry = g;
  return FVC_OK;
}

int32_t fvc_cells_geometry_destroy(void *geometry) {
  if (geometry) cudaFree(geometry);
  return FVC_OK;
}

}  // extern "C"
