/*
 * fvc_oracle.c -- CPU restatement of the fortranFVCell linear-solver hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for libfvcgpu and the timed
 * CPU baseline of bench.py.  The product never links or calls this file.
 *
 * Each function restates the cited Fortran routine with its loop order and
 * 1-based index semantics.  Fortran array a(i) is written F1(a,i); a 2-D
 * Fortran array a(d1,*) element a(i,j) is F2(a,d1,i,j).
 * Parity status: partially pinned (reference dot KAT + hand-derived cases);
 * the reference itself cannot be compiled here (Fortran, no compiler).
 */
#include "fvc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define F1(a, i) ((a)[(i)-1])
#define F2(a, d1, i, j) ((a)[((i)-1) + (size_t)((j)-1) * (size_t)(d1)])

/* ======================================================================
 * Adjacency: src/Adjacency.f:1-94 (adjtria3) and :95-189 (adjquad4).
 * The two differ only in the number of sides and in the claim test of the
 * first sweep: adjtria3 claims an edge when BOTH end nodes are free
 * (.and., :49), adjquad4 when EITHER is free (.or., :143).
 * ====================================================================== */
static void adj_generic(const int32_t *ix, int32_t *nodcon, int32_t *nelcon,
                        int32_t nnode, int32_t numel, int32_t nen, int32_t ns,
                        int use_or, int32_t *nedge) {
  static const int32_t isnod3[2 * 3] = {1, 2, 2, 3, 3, 1};
  static const int32_t isnod4[2 * 4] = {1, 2, 2, 3, 3, 4, 4, 1};
  const int32_t *isnod = (ns == 3) ? isnod3 : isnod4;
  const int32_t ldx = nen + 1;
  int32_t nel, is, no, imiss, no1, no2, nel2, is2, no21, no22;
  *nedge = 0;
  for (nel = 1; nel <= numel; ++nel)
    for (is = 1; is <= ns; ++is) F2(nelcon, ns, is, nel) = 0;
  for (no = 1; no <= nnode; ++no) F1(nodcon, no) = 0;
  do {
    imiss = 0;
    for (nel = 1; nel <= numel; ++nel)
      for (is = 1; is <= ns; ++is) {
        if (F2(nelcon, ns, is, nel) != 0) continue;
        no1 = F2(ix, ldx, F2(isnod, 2, 1, is), nel);
        no2 = F2(ix, ldx, F2(isnod, 2, 2, is), nel);
        int claim = use_or ? (F1(nodcon, no1) == 0 || F1(nodcon, no2) == 0)
                           : (F1(nodcon, no1) == 0 && F1(nodcon, no2) == 0);
        if (claim) {
          F1(nodcon, no1) = nel;
          F1(nodcon, no2) = nel;
          imiss = 1;
        }
      }
    for (nel = 1; nel <= numel; ++nel)
      for (is = 1; is <= ns; ++is) {
        if (F2(nelcon, ns, is, nel) != 0) continue;
        no1 = F2(ix, ldx, F2(isnod, 2, 1, is), nel);
        no2 = F2(ix, ldx, F2(isnod, 2, 2, is), nel);
        nel2 = F1(nodcon, no1);
        if (nel2 > 0) {
          if (nel2 == F1(nodcon, no2) && nel2 != nel) {
            for (is2 = 1; is2 <= ns; ++is2) {
              no21 = F2(ix, ldx, F2(isnod, 2, 1, is2), nel2);
              no22 = F2(ix, ldx, F2(isnod, 2, 2, is2), nel2);
              if (no21 == no2 && no22 == no1) {
                F2(nelcon, ns, is, nel) = nel2;
                F2(nelcon, ns, is2, nel2) = nel;
                F1(nodcon, no1) = 0;
                F1(nodcon, no2) = 0;
                imiss = 1;
                *nedge += 1;
              }
            }
          }
        }
      }
    for (nel = 1; nel <= numel; ++nel)
      for (is = 1; is <= ns; ++is) {
        if (F2(nelcon, ns, is, nel) != 0) continue;
        no1 = F2(ix, ldx, F2(isnod, 2, 1, is), nel);
        no2 = F2(ix, ldx, F2(isnod, 2, 2, is), nel);
        if (F1(nodcon, no1) == F1(nodcon, no2) && F1(nodcon, no1) == nel) {
          F2(nelcon, ns, is, nel) = -1;
          F1(nodcon, no1) = 0;
          F1(nodcon, no2) = 0;
          imiss = 1;
          *nedge += 1;
        }
      }
  } while (imiss == 1);
}

void oref_adjtria3(const int32_t *ix, int32_t *nodcon, int32_t *nelcon,
                   int32_t nnode, int32_t numel, int32_t nen, int32_t *nedge) {
  adj_generic(ix, nodcon, nelcon, nnode, numel, nen, 3, 0, nedge);
}

void oref_adjquad4(const int32_t *ix, int32_t *nodcon, int32_t *nelcon,
                   int32_t nnode, int32_t numel, int32_t nen, int32_t *nedge) {
  adj_generic(ix, nodcon, nelcon, nnode, numel, nen, 4, 1, nedge);
  *nedge += 2 * numel; /* Adjacency.f:186 */
}

/* adjquad4's sweeps generalised to meshes mixing triangles and quads (the
 * reference has no such path): a cell's side count is its number of
 * nonzero node slots (ix(ld,numel), 1-based nodes, 0 = unused); unused
 * sides get -1.  For one-type meshes the result equals adjtria3/adjquad4. */
void oref_adjacency_mixed(const int32_t *ix, int32_t ld, int32_t *nodcon, int32_t *nelcon,
                          int32_t nnode, int32_t numel, int32_t nshared) {
  int32_t nel, is, no, imiss, no1, no2, nel2, is2;
  int32_t *ns = (int32_t *)malloc(sizeof(int32_t) * (size_t)numel);
  for (nel = 1; nel <= numel; ++nel) {
    int32_t c = 0;
    while (c < nshared && c < ld && F2(ix, ld, c + 1, nel) > 0) c++;
    F1(ns, nel) = c;
    for (is = 1; is <= nshared; ++is) F2(nelcon, nshared, is, nel) = (is <= c) ? 0 : -1;
  }
  for (no = 1; no <= nnode; ++no) F1(nodcon, no) = 0;
#define SIDE_NODES(cell, side, a, b)                                     \
  do {                                                                   \
    a = F2(ix, ld, side, cell);                                          \
    b = F2(ix, ld, (side % F1(ns, cell)) + 1, cell);                     \
  } while (0)
  do {
    imiss = 0;
    for (nel = 1; nel <= numel; ++nel)
      for (is = 1; is <= F1(ns, nel); ++is) {
        if (F2(nelcon, nshared, is, nel) != 0) continue;
        SIDE_NODES(nel, is, no1, no2);
        if (F1(nodcon, no1) == 0 || F1(nodcon, no2) == 0) {
          F1(nodcon, no1) = nel;
          F1(nodcon, no2) = nel;
          imiss = 1;
        }
      }
    for (nel = 1; nel <= numel; ++nel)
      for (is = 1; is <= F1(ns, nel); ++is) {
        if (F2(nelcon, nshared, is, nel) != 0) continue;
        SIDE_NODES(nel, is, no1, no2);
        nel2 = F1(nodcon, no1);
        if (nel2 > 0 && nel2 == F1(nodcon, no2) && nel2 != nel) {
          for (is2 = 1; is2 <= F1(ns, nel2); ++is2) {
            int32_t no21, no22;
            SIDE_NODES(nel2, is2, no21, no22);
            if (no21 == no2 && no22 == no1) {
              F2(nelcon, nshared, is, nel) = nel2;
              F2(nelcon, nshared, is2, nel2) = nel;
              F1(nodcon, no1) = 0;
              F1(nodcon, no2) = 0;
              imiss = 1;
            }
          }
        }
      }
    for (nel = 1; nel <= numel; ++nel)
      for (is = 1; is <= F1(ns, nel); ++is) {
        if (F2(nelcon, nshared, is, nel) != 0) continue;
        SIDE_NODES(nel, is, no1, no2);
        if (F1(nodcon, no1) == F1(nodcon, no2) && F1(nodcon, no1) == nel) {
          F2(nelcon, nshared, is, nel) = -1;
          F1(nodcon, no1) = 0;
          F1(nodcon, no2) = 0;
          imiss = 1;
        }
      }
  } while (imiss == 1);
#undef SIDE_NODES
  free(ns);
}

/* ======================================================================
 * RCM: src/Reord.f (SPARSPAK genrcm/fnroot/rcm/rootls/degree) and
 * src/Graph.f:18-41 (conv_graph).
 * ====================================================================== */
static void conv_graph(const int32_t *viz, int32_t numel, int32_t nshared,
                       int32_t *xadj, int32_t *adjncy) {
  /* Graph.f:18-41 */
  F1(xadj, 1) = 1;
  for (int32_t i = 1; i <= numel; ++i) {
    int32_t aux = 0, ipont = F1(xadj, i);
    for (int32_t j = 1; j <= nshared; ++j) {
      int32_t nelviz = F2(viz, nshared, j, i);
      if (nelviz != -1) {
        F1(adjncy, ipont + aux) = nelviz;
        aux++;
      }
    }
    F1(xadj, i + 1) = F1(xadj, i) + aux;
  }
}

static void rootls(int32_t root, const int32_t *xadj, const int32_t *adjncy,
                   int32_t *mask, int32_t *nlvl, int32_t *xls, int32_t *ls) {
  /* Reord.f:294-357 */
  int32_t i, j, jstop, jstrt, lbegin, ccsize, lvlend, lvsize, nbr, node;
  F1(mask, root) = 0;
  F1(ls, 1) = root;
  *nlvl = 0;
  lvlend = 0;
  ccsize = 1;
  do {
    lbegin = lvlend + 1;
    lvlend = ccsize;
    *nlvl += 1;
    F1(xls, *nlvl) = lbegin;
    for (i = lbegin; i <= lvlend; ++i) {
      node = F1(ls, i);
      jstrt = F1(xadj, node);
      jstop = F1(xadj, node + 1) - 1;
      for (j = jstrt; j <= jstop; ++j) {
        nbr = F1(adjncy, j);
        if (F1(mask, nbr) == 0) continue;
        ccsize++;
        F1(ls, ccsize) = nbr;
        F1(mask, nbr) = 0;
      }
    }
    lvsize = ccsize - lvlend;
  } while (lvsize > 0);
  F1(xls, *nlvl + 1) = lvlend + 1;
  for (i = 1; i <= ccsize; ++i) F1(mask, F1(ls, i)) = 1;
}

static void fnroot(int32_t *root, const int32_t *xadj, const int32_t *adjncy,
                   int32_t *mask, int32_t *nlvl, int32_t *xls, int32_t *ls) {
  /* Reord.f:112-164.  Note the reference's ".ge." in the last-level scan
   * (Reord.f:145), kept as is: it changes which root is chosen. */
  int32_t ccsize, j, jstrt, k, kstop, kstrt, mindeg, nabor, ndeg, node, nunlvl;
  rootls(*root, xadj, adjncy, mask, nlvl, xls, ls);
  ccsize = F1(xls, *nlvl + 1) - 1;
  if (*nlvl == 1 || *nlvl == ccsize) return;
  for (;;) {
    jstrt = F1(xls, *nlvl);
    mindeg = ccsize;
    *root = F1(ls, jstrt);
    if (ccsize != jstrt) {
      for (j = jstrt; j <= ccsize; ++j) {
        node = F1(ls, j);
        ndeg = 0;
        kstrt = F1(xadj, node);
        kstop = F1(xadj, node + 1) - 1;
        for (k = kstrt; k <= kstop; ++k) {
          nabor = F1(adjncy, k);
          if (F1(mask, nabor) > 0) ndeg++;
        }
        if (ndeg >= mindeg) {
          *root = node;
          mindeg = ndeg;
        }
      }
    }
    rootls(*root, xadj, adjncy, mask, &nunlvl, xls, ls);
    if (nunlvl <= *nlvl) return;
    *nlvl = nunlvl;
    if (*nlvl >= ccsize) return;
  }
}

static void degree(int32_t root, int32_t *xadj, const int32_t *adjncy,
                   const int32_t *mask, int32_t *deg, int32_t *ccsize,
                   int32_t *ls) {
  /* Reord.f:358-457: xadj entries are negated as visit markers */
  int32_t i, j, jstop, jstrt, lbegin, lvlend, lvsize, nbr, ideg, node;
  F1(ls, 1) = root;
  F1(xadj, root) = -F1(xadj, root);
  lvlend = 0;
  *ccsize = 1;
  do {
    lbegin = lvlend + 1;
    lvlend = *ccsize;
    for (i = lbegin; i <= lvlend; ++i) {
      node = F1(ls, i);
      jstrt = -F1(xadj, node);
      jstop = abs(F1(xadj, node + 1)) - 1;
      ideg = 0;
      for (j = jstrt; j <= jstop; ++j) {
        nbr = F1(adjncy, j);
        if (F1(mask, nbr) == 0) continue;
        ideg++;
        if (F1(xadj, nbr) < 0) continue;
        F1(xadj, nbr) = -F1(xadj, nbr);
        *ccsize += 1;
        F1(ls, *ccsize) = nbr;
      }
      F1(deg, node) = ideg;
    }
    lvsize = *ccsize - lvlend;
  } while (lvsize > 0);
  for (i = 1; i <= *ccsize; ++i) {
    node = F1(ls, i);
    F1(xadj, node) = -F1(xadj, node);
  }
}

static void rcm(int32_t root, int32_t *xadj, const int32_t *adjncy,
                int32_t *mask, int32_t *perm, int32_t *ccsize, int32_t *deg) {
  /* Reord.f:165-293 */
  int32_t fnbr, i, j, jstop, jstrt, k, l, lbegin, lnbr, lperm, lvlend, nbr,
      node;
  degree(root, xadj, adjncy, mask, deg, ccsize, perm);
  F1(mask, root) = 0;
  if (*ccsize <= 1) return;
  lvlend = 0;
  lnbr = 1;
  do {
    lbegin = lvlend + 1;
    lvlend = lnbr;
    for (i = lbegin; i <= lvlend; ++i) {
      node = F1(perm, i);
      jstrt = F1(xadj, node);
      jstop = F1(xadj, node + 1) - 1;
      fnbr = lnbr + 1;
      for (j = jstrt; j <= jstop; ++j) {
        nbr = F1(adjncy, j);
        if (F1(mask, nbr) != 0) {
          lnbr++;
          F1(mask, nbr) = 0;
          F1(perm, lnbr) = nbr;
        }
      }
      if (fnbr < lnbr) {
        /* linear insertion sort of the new neighbours by degree */
        k = fnbr;
        do {
          l = k;
          k = k + 1;
          nbr = F1(perm, k);
          while (l >= fnbr) {
            lperm = F1(perm, l);
            if (F1(deg, lperm) <= F1(deg, nbr)) break;
            F1(perm, l + 1) = lperm;
            l = l - 1;
          }
          F1(perm, l + 1) = nbr;
        } while (k < lnbr);
      }
    }
  } while (lnbr > lvlend);
  k = *ccsize / 2;
  l = *ccsize;
  for (i = 1; i <= k; ++i) {
    lperm = F1(perm, l);
    F1(perm, l) = F1(perm, i);
    F1(perm, i) = lperm;
    l = l - 1;
  }
}

static void genrcm(int32_t neq, int32_t *xadj, const int32_t *adjncy,
                   int32_t *perm, int32_t *mask, int32_t *xls) {
  /* Reord.f:53-111 */
  int32_t ccsize, i, nlvl, num, root;
  for (i = 1; i <= neq; ++i) F1(mask, i) = 1;
  num = 1;
  for (i = 1; i <= neq; ++i) {
    if (F1(mask, i) != 0) {
      root = i;
      fnroot(&root, xadj, adjncy, mask, &nlvl, xls, &F1(perm, num));
      rcm(root, xadj, adjncy, mask, &F1(perm, num), &ccsize, xls);
      num += ccsize;
      if (neq < num) return;
    }
  }
}

void oref_reord(const int32_t *viz, int32_t *iperm, int32_t numel,
                int32_t nshared, int32_t alf) {
  /* Reord.f:6-52 */
  if (alf) {
    int32_t *xadj = (int32_t *)calloc((size_t)numel + 1, sizeof(int32_t));
    int32_t *adjncy =
        (int32_t *)calloc((size_t)nshared * numel + 1, sizeof(int32_t));
    int32_t *mask = (int32_t *)calloc((size_t)numel + 1, sizeof(int32_t));
    int32_t *xls = (int32_t *)calloc((size_t)numel + 2, sizeof(int32_t));
    int32_t *perm = (int32_t *)calloc((size_t)numel + 1, sizeof(int32_t));
    conv_graph(viz, numel, nshared, xadj, adjncy);
    memset(iperm, 0, sizeof(int32_t) * (size_t)numel);
    genrcm(numel, xadj, adjncy, perm, mask, xls);
    for (int32_t i = 1; i <= numel; ++i) F1(iperm, F1(perm, i)) = i;
    free(xadj);
    free(adjncy);
    free(mask);
    free(xls);
    free(perm);
  } else {
    for (int32_t i = 1; i <= numel; ++i) F1(iperm, i) = i;
  }
}

/* ======================================================================
 * Equation numbering and sparse structures
 * ====================================================================== */
void oref_numeq(int32_t *id, const int32_t *num, const int32_t *elconn,
                int32_t numel, int32_t nshared, int32_t *neq) {
  /* Numeq.f:4-25 */
  *neq = numel;
  for (int32_t i = 1; i <= numel; ++i) {
    int32_t n = F1(num, i);
    for (int32_t j = 1; j <= nshared; ++j) {
      int32_t nelviz = F2(elconn, nshared, j, i);
      F2(id, nshared, j, n) = (nelviz != -1) ? F1(num, nelviz) : -1;
    }
  }
}

void oref_csria(int32_t *ia, const int32_t *id, int32_t neq, int32_t nshared,
                int32_t *nad, int32_t upper, int32_t lower, int32_t diag) {
  /* Csr.f:21-55 */
  F1(ia, 1) = 1;
  for (int32_t i = 1; i <= neq; ++i) {
    int32_t aux = 0;
    for (int32_t j = 1; j <= nshared; ++j) {
      int32_t nl = F2(id, nshared, j, i);
      if (nl != -1) {
        if (lower && nl < i)
          aux++;
        else if (upper && nl > i)
          aux++;
      }
    }
    if (diag) aux++;
    F1(ia, i + 1) = F1(ia, i) + aux;
  }
  *nad = F1(ia, neq + 1) - F1(ia, 1);
}

void oref_csrja(const int32_t *ia, int32_t *ja, const int32_t *id, int32_t neq,
                int32_t nshared, int32_t upper, int32_t lower, int32_t diag) {
  /* Csr.f:76-110 */
  for (int32_t i = 1; i <= neq; ++i) {
    int32_t aux = 0, ipont = F1(ia, i);
    if (diag) {
      F1(ja, ipont + aux) = i;
      aux++;
    }
    for (int32_t j = 1; j <= nshared; ++j) {
      int32_t nl = F2(id, nshared, j, i);
      if (nl != -1) {
        if (nl < i && lower) {
          F1(ja, ipont + aux) = nl;
          aux++;
        } else if (nl > i && upper) {
          F1(ja, ipont + aux) = nl;
          aux++;
        }
      }
    }
  }
}

static void bubblesort(int32_t *ja, int32_t n) {
  /* Graph.f:71-93 */
  int32_t itroca;
  do {
    itroca = 0;
    for (int32_t i = 2; i <= n; ++i) {
      if (F1(ja, i) < F1(ja, i - 1)) {
        int32_t j = F1(ja, i - 1);
        F1(ja, i - 1) = F1(ja, i);
        F1(ja, i) = j;
        itroca = 1;
      }
    }
  } while (itroca == 1);
}

void oref_sortgraph(const int32_t *ia, int32_t *ja, int32_t neq) {
  /* Graph.f:45-70 */
  for (int32_t i = 1; i <= neq; ++i)
    bubblesort(&F1(ja, F1(ia, i)), F1(ia, i + 1) - F1(ia, i));
}

void oref_ellpackja(int32_t *ifellpack, int32_t *ja, const int32_t *id,
                    int32_t neq, int32_t *nad, int32_t nshared) {
  /* EllPack.f:19-42 */
  F1(ifellpack, 1) = nshared;
  F1(ifellpack, 2) = neq + 1;
  *nad = 0;
  for (int32_t i = 1; i <= neq; ++i)
    for (int32_t j = 1; j <= nshared; ++j) {
      int32_t nl = F2(id, nshared, j, i);
      if (nl == -1) {
        F2(ja, nshared, j, i) = 1;
      } else {
        *nad += 1;
        F2(ja, nshared, j, i) = nl;
      }
    }
}

int32_t oref_banda_csr(const int32_t *ia, const int32_t *ja, int32_t neq) {
  /* Csr.f:245-272 (colMax starts at 0; the reference leaves it undefined
   * on the first row) */
  int32_t bandmax = 0, colmax = 0;
  for (int32_t i = 1; i <= neq; ++i) {
    for (int32_t j = F1(ia, i); j <= F1(ia, i + 1) - 1; ++j) {
      int32_t col = abs(i - F1(ja, j));
      if (col > colmax) colmax = col;
    }
    if (colmax > bandmax) bandmax = colmax;
    colmax = 0;
  }
  return bandmax;
}

int32_t oref_datastruc(const int32_t *id, int32_t *ia, int32_t *ja, int32_t neq,
                       int32_t nshared, int32_t matriz, int32_t unsym) {
  /* Datastruct.f:27-179, structure part only */
  int32_t nad = 0, upper = 0, lower = 0, diag = 0;
  if (matriz == 4) {
    if (ja == NULL) return nshared * neq;
    oref_ellpackja(ia, ja, id, neq, &nad, nshared);
    return nad;
  }
  if (matriz == 1) {
    lower = 1;
    upper = unsym ? 1 : 0;
    diag = 0;
  } else if (matriz == 2) {
    upper = lower = diag = 1;
  } else if (matriz == 3) {
    upper = 0;
    lower = 1;
    diag = 0;
  } else {
    return -1;
  }
  oref_csria(ia, id, neq, nshared, &nad, upper, lower, diag);
  if (ja == NULL) return nad;
  oref_csrja(ia, ja, id, neq, nshared, upper, lower, diag);
  if (matriz != 2) oref_sortgraph(ia, ja, neq);
  return nad;
}

/* ======================================================================
 * Assembly scatter: src/Assbly.f:32-54, src/Csr.f:142-227,
 * src/EllPack.f:68-93.  Off-diagonals are stored negated.
 * ====================================================================== */
void oref_assbly(double *ad, double *au, double *al, double *f,
                 const int32_t *ia, const int32_t *ja, const double *la,
                 double p, const int32_t *ld, int32_t nshared, int32_t cod,
                 int32_t unsym, int32_t forces, int32_t matrix) {
  (void)unsym;
  int32_t n = F1(ld, nshared + 1);
  if (cod == 1) {
    if (matrix) F1(ad, n) = F1(la, nshared + 1);
    if (forces) F1(f, n) = p;
    int32_t ipont = F1(ia, n), iak = F1(ia, n + 1) - F1(ia, n);
    if (matrix)
      for (int32_t j = 1; j <= nshared; ++j) {
        int32_t l = F1(ld, j);
        if (l > 0)
          for (int32_t i = 1; i <= iak; ++i) {
            int32_t k = ipont + i - 1;
            if (l == F1(ja, k)) F1(au, k) = -F1(la, j);
          }
      }
  } else if (cod == 2) {
    if (forces) F1(f, n) = p;
    int32_t ipont = F1(ia, n), iak = F1(ia, n + 1) - F1(ia, n);
    for (int32_t j = 1; j <= nshared + 1; ++j) {
      int32_t l = F1(ld, j);
      if (l > 0)
        for (int32_t i = 1; i <= iak; ++i) {
          int32_t k = ipont + i - 1;
          if (l == F1(ja, k) && matrix) F1(ad, k) = -F1(la, j);
        }
    }
  } else if (cod == 3) {
    F1(ad, n) = F1(la, nshared + 1);
    if (forces) F1(f, n) = p;
    int32_t ipont = F1(ia, n), iak = F1(ia, n + 1) - F1(ia, n);
    for (int32_t j = 1; j <= nshared; ++j) {
      int32_t l = F1(ld, j);
      if (l > 0)
        for (int32_t i = 1; i <= iak; ++i) {
          int32_t k = ipont + i - 1;
          if (l == F1(ja, k) && matrix) F1(al, k) = -F1(la, j);
        }
    }
  } else if (cod == 4) {
    /* EllPack.f:68-93: values go to the al slice */
    if (forces) F1(f, n) = p;
    if (matrix) {
      F1(ad, n) = F1(la, nshared + 1);
      for (int32_t j = 1; j <= nshared; ++j) {
        int32_t l = F1(ld, j);
        F2(al, nshared, j, n) = (l > 0) ? -F1(la, j) : 0.0;
      }
    }
  }
}

/* ======================================================================
 * SpMV + BLAS-1: src/Matvec.f
 * ====================================================================== */
void oref_matvec_csrd(const double *ad, const double *a, const double *dum,
                      const double *x, double *y, const int32_t *ia,
                      const int32_t *ja, int32_t neq) {
  /* Matvec.f:21-39 */
  (void)dum;
  for (int32_t i = 1; i <= neq; ++i) {
    double t = F1(ad, i) * F1(x, i);
    for (int32_t j = F1(ia, i); j <= F1(ia, i + 1) - 1; ++j)
      t = t + F1(a, j) * F1(x, F1(ja, j));
    F1(y, i) = t;
  }
}

void oref_matvec_csr(const double *a, const double *d1, const double *d2,
                     const double *x, double *y, const int32_t *ia,
                     const int32_t *ja, int32_t neq) {
  /* Matvec.f:61-78 */
  (void)d1;
  (void)d2;
  for (int32_t i = 1; i <= neq; ++i) {
    double t = 0.0;
    for (int32_t j = F1(ia, i); j <= F1(ia, i + 1) - 1; ++j)
      t = t + F1(a, j) * F1(x, F1(ja, j));
    F1(y, i) = t;
  }
}

void oref_matvec_csrc(const double *ad, const double *au, const double *al,
                      const double *x, double *y, const int32_t *ia,
                      const int32_t *ja, int32_t neq) {
  /* Matvec.f:102-135 */
  for (int32_t i = 1; i <= neq; ++i) {
    double xi = F1(x, i);
    double t = F1(ad, i) * xi;
    for (int32_t k = F1(ia, i); k <= F1(ia, i + 1) - 1; ++k) {
      int32_t jak = F1(ja, k);
      t = t + F1(al, k) * F1(x, jak);
      F1(y, jak) = F1(y, jak) + F1(au, k) * xi;
    }
    F1(y, i) = t;
  }
}

void oref_matvec_csrc_sym(const double *ad, const double *dum, const double *al,
                          const double *x, double *y, const int32_t *ia,
                          const int32_t *ja, int32_t neq) {
  /* Matvec.f:157-192 */
  (void)dum;
  F1(y, 1) = F1(ad, 1) * F1(x, 1);
  for (int32_t i = 2; i <= neq; ++i) {
    double xi = F1(x, i);
    double t = F1(ad, i) * xi;
    for (int32_t k = F1(ia, i); k <= F1(ia, i + 1) - 1; ++k) {
      int32_t jak = F1(ja, k);
      double s = F1(al, k);
      t = t + s * F1(x, jak);
      F1(y, jak) = F1(y, jak) + s * xi;
    }
    F1(y, i) = t;
  }
}

void oref_matvec_csrd_sym(const double *ad, const double *dum, const double *al,
                          const double *x, double *y, const int32_t *ia,
                          const int32_t *ja, int32_t neq) {
  /* Matvec.f:216-250 (same loop as csrc_sym) */
  oref_matvec_csrc_sym(ad, dum, al, x, y, ia, ja, neq);
}

void oref_matvec_ellpack(const double *ad, const double *a, const double *dum,
                         const double *x, double *y, const int32_t *nl,
                         const int32_t *ja, int32_t neq) {
  /* Matvec.f:271-300: widths 3 and 4 only */
  (void)dum;
  int32_t w = F1(nl, 1);
  if (w == 3) {
    for (int32_t i = 1; i <= neq; ++i) {
      double t4 = F1(ad, i) * F1(x, i);
      double t1 = F2(a, 3, 1, i) * F1(x, F2(ja, 3, 1, i));
      double t2 = F2(a, 3, 2, i) * F1(x, F2(ja, 3, 2, i));
      double t3 = F2(a, 3, 3, i) * F1(x, F2(ja, 3, 3, i));
      F1(y, i) = t1 + t2 + t3 + t4;
    }
  } else if (w == 4) {
    for (int32_t i = 1; i <= neq; ++i) {
      double t5 = F1(ad, i) * F1(x, i);
      double t1 = F2(a, 4, 1, i) * F1(x, F2(ja, 4, 1, i));
      double t2 = F2(a, 4, 2, i) * F1(x, F2(ja, 4, 2, i));
      double t3 = F2(a, 4, 3, i) * F1(x, F2(ja, 4, 3, i));
      double t4 = F2(a, 4, 4, i) * F1(x, F2(ja, 4, 4, i));
      F1(y, i) = t1 + t2 + t3 + t4 + t5;
    }
  }
}

double oref_dot(const double *a, const double *b, int32_t n) {
  /* Matvec.f:383-402 */
  double d = 0.0;
  for (int32_t i = 1; i <= n; ++i) d = d + F1(a, i) * F1(b, i);
  return d;
}

double oref_smachn(void) {
  /* Iterativos.f:450-462 */
  volatile double s = 1.0;
  do {
    s = s * 0.5;
  } while (s + 1.0 != 1.0);
  return s;
}

void oref_getres(double *u, double *x, const int32_t *num, int32_t neq,
                 int32_t numel, int32_t flag) {
  /* Solver.f:368-391 */
  (void)neq;
  if (flag)
    for (int32_t i = 1; i <= numel; ++i) F1(x, F1(num, i)) = F1(u, i);
  else
    for (int32_t i = 1; i <= numel; ++i) F1(u, i) = F1(x, F1(num, i));
}

/* ======================================================================
 * Sequential Krylov solvers: src/Iterativos.f
 * ====================================================================== */
typedef void (*matvec_fn)(const double *, const double *, const double *,
                          const double *, double *, const int32_t *,
                          const int32_t *, int32_t);

static int32_t pcg(int32_t neq, const int32_t *ia, const int32_t *ja,
                   const double *ad, const double *au, const double *al,
                   const double *m, double *b, double *x, double *z, double *r,
                   double tol, int32_t maxit, matvec_fn matvec, int32_t init,
                   oref_stats *st) {
  /* Iterativos.f:29-106 */
  double d, conv, alpha, beta;
  int32_t i, j;
  if (init)
    for (i = 1; i <= neq; ++i) F1(x, i) = 0.0;
  matvec(ad, au, al, x, z, ia, ja, neq);
  for (i = 1; i <= neq; ++i) {
    F1(r, i) = F1(b, i) - F1(z, i);
    F1(z, i) = F1(r, i) / F1(m, i);
    F1(b, i) = F1(z, i);
  }
  d = oref_dot(r, z, neq);
  conv = tol * sqrt(fabs(d));
  st->conv = conv;
  for (j = 1; j <= maxit; ++j) {
    matvec(ad, au, al, b, z, ia, ja, neq);
    alpha = d / oref_dot(b, z, neq);
    for (i = 1; i <= neq; ++i) {
      F1(x, i) = F1(x, i) + alpha * F1(b, i);
      F1(r, i) = F1(r, i) - alpha * F1(z, i);
      F1(z, i) = F1(r, i) / F1(m, i);
    }
    beta = oref_dot(r, z, neq) / d;
    for (i = 1; i <= neq; ++i) F1(b, i) = F1(z, i) + beta * F1(b, i);
    d = beta * d;
    if (sqrt(fabs(d)) < conv) break;
  }
  st->final_crit = sqrt(fabs(d));
  if (j > maxit) {
    st->iterations = maxit;
    st->status = OREF_NOCONV;
    return OREF_NOCONV;
  }
  st->iterations = j;
  matvec(ad, au, al, x, z, ia, ja, neq);
  st->energy = oref_dot(x, z, neq);
  st->status = OREF_OK;
  return OREF_OK;
}

static int32_t pbicgstab(int32_t neq, const int32_t *ia, const int32_t *ja,
                         const double *ad, const double *au, const double *al,
                         const double *m, double *b, double *x, double *t,
                         double *v, double *r, double *p, double *z, double tol,
                         int32_t maxit, matvec_fn matvec, int32_t init,
                         oref_stats *st) {
  /* Iterativos.f:140-234 */
  double conv, d, alpha, beta, rr0, w;
  int32_t i, j;
  if (init)
    for (i = 1; i <= neq; ++i) F1(x, i) = 0.0;
  matvec(ad, au, al, x, z, ia, ja, neq);
  for (i = 1; i <= neq; ++i) {
    F1(r, i) = F1(b, i) - F1(z, i);
    F1(p, i) = F1(r, i);
    F1(b, i) = F1(p, i);
    F1(z, i) = F1(p, i) / F1(m, i);
  }
  d = oref_dot(r, z, neq);
  conv = tol * sqrt(fabs(d));
  st->conv = conv;
  beta = 0.0;
  for (j = 1; j <= maxit; ++j) {
    matvec(ad, au, al, z, v, ia, ja, neq);
    rr0 = oref_dot(b, r, neq);
    alpha = rr0 / oref_dot(v, r, neq);
    for (i = 1; i <= neq; ++i) {
      F1(x, i) = F1(x, i) + alpha * F1(z, i);
      F1(b, i) = F1(b, i) - alpha * F1(v, i);
      F1(z, i) = F1(b, i) / F1(m, i);
    }
    matvec(ad, au, al, z, t, ia, ja, neq);
    w = oref_dot(t, b, neq) / oref_dot(t, t, neq);
    for (i = 1; i <= neq; ++i) {
      F1(x, i) = F1(x, i) + w * F1(z, i);
      F1(b, i) = F1(b, i) - w * F1(t, i);
    }
    beta = oref_dot(b, z, neq) / d;
    if (sqrt(fabs(beta)) < conv) break;
    beta = (oref_dot(r, b, neq) / rr0) * (alpha / w);
    for (i = 1; i <= neq; ++i) {
      F1(p, i) = F1(b, i) + beta * (F1(p, i) - w * F1(v, i));
      F1(z, i) = F1(p, i) / F1(m, i);
    }
  }
  st->final_crit = sqrt(fabs(beta));
  if (j > maxit) {
    st->iterations = maxit;
    st->status = OREF_NOCONV;
    return OREF_NOCONV;
  }
  st->iterations = j;
  matvec(ad, au, al, x, z, ia, ja, neq);
  st->energy = oref_dot(x, z, neq);
  st->status = OREF_OK;
  return OREF_OK;
}

static int32_t gmres(int32_t neq, const int32_t *ia, const int32_t *ja,
                     const double *ad, const double *au, const double *al,
                     const double *m, const double *b, double *x, int32_t k,
                     double *g, double *h, double *y, double *c, double *s,
                     double *e, double tol, int32_t maxit, matvec_fn matvec,
                     oref_stats *st) {
  /* Iterativos.f:271-446.  g(neq,k+1), h(k+1,k) */
  double econv, norm, r, aux1, aux2, beta;
  int32_t nit, i, j, l, ni = 0, ic;
  for (i = 1; i <= neq; ++i) F1(x, i) = 0.0;
  norm = sqrt(oref_dot(b, b, neq));
  econv = tol * norm;
  st->conv = econv;
  nit = 0;
  for (l = 1; l <= maxit; ++l) {
    matvec(ad, au, al, x, g, ia, ja, neq);
    for (i = 1; i <= neq; ++i)
      F2(g, neq, i, 1) = (F1(b, i) - F2(g, neq, i, 1)) / F1(m, i);
    F1(e, 1) = sqrt(oref_dot(g, g, neq));
    for (i = 1; i <= neq; ++i) F2(g, neq, i, 1) = F2(g, neq, i, 1) / F1(e, 1);
    ni = 0;
    for (i = 1; i <= k; ++i) {
      nit++;
      ni++;
      matvec(ad, au, al, &F2(g, neq, 1, i), &F2(g, neq, 1, i + 1), ia, ja, neq);
      for (j = 1; j <= neq; ++j)
        F2(g, neq, j, i + 1) = F2(g, neq, j, i + 1) / F1(m, j);
      for (j = 1; j <= i; ++j) {
        beta = oref_dot(&F2(g, neq, 1, i + 1), &F2(g, neq, 1, j), neq);
        for (ic = 1; ic <= neq; ++ic)
          F2(g, neq, ic, i + 1) = F2(g, neq, ic, i + 1) - beta * F2(g, neq, ic, j);
        F2(h, k + 1, j, i) = beta;
      }
      norm = sqrt(oref_dot(&F2(g, neq, 1, i + 1), &F2(g, neq, 1, i + 1), neq));
      F2(h, k + 1, i + 1, i) = norm;
      for (ic = 1; ic <= neq; ++ic)
        F2(g, neq, ic, i + 1) = F2(g, neq, ic, i + 1) / norm;
      for (j = 1; j <= i - 1; ++j) {
        aux1 = F1(c, j) * F2(h, k + 1, j, i) + F1(s, j) * F2(h, k + 1, j + 1, i);
        aux2 = -F1(s, j) * F2(h, k + 1, j, i) + F1(c, j) * F2(h, k + 1, j + 1, i);
        F2(h, k + 1, j, i) = aux1;
        F2(h, k + 1, j + 1, i) = aux2;
      }
      r = sqrt(F2(h, k + 1, i, i) * F2(h, k + 1, i, i) +
               F2(h, k + 1, i + 1, i) * F2(h, k + 1, i + 1, i));
      F1(c, i) = F2(h, k + 1, i, i) / r;
      F1(s, i) = F2(h, k + 1, i + 1, i) / r;
      F2(h, k + 1, i, i) = r;
      F2(h, k + 1, i + 1, i) = 0.0;
      F1(e, i + 1) = -F1(s, i) * F1(e, i);
      F1(e, i) = F1(c, i) * F1(e, i);
      if (fabs(F1(e, i + 1)) <= econv) break;
    }
    F1(y, ni) = F1(e, ni) / F2(h, k + 1, ni, ni);
    for (i = ni - 1; i >= 1; --i) {
      F1(y, i) = 0.0;
      for (j = i + 1; j <= ni; ++j)
        F1(y, i) = F1(y, i) - F2(h, k + 1, i, j) * F1(y, j);
      F1(y, i) = (F1(y, i) + F1(e, i)) / F2(h, k + 1, i, i);
    }
    for (i = 1; i <= neq; ++i)
      for (j = 1; j <= ni; ++j) F1(x, i) = F1(x, i) + F1(y, j) * F2(g, neq, i, j);
    if (fabs(F1(e, ni + 1)) <= econv) break;
  }
  st->inner_its = nit;
  st->final_crit = fabs(F1(e, ni + 1));
  if (l > maxit) {
    st->iterations = maxit;
    st->status = OREF_NOCONV;
    return OREF_NOCONV;
  }
  st->iterations = l;
  st->energy = oref_dot(x, b, neq);
  st->status = OREF_OK;
  return OREF_OK;
}

/* ======================================================================
 * OpenMP variants: src/Matvec_omp.f and src/Iterativos_omp.f.
 * These run inside one parallel region with orphaned worksharing loops.
 * The dot accumulators are shared (the reference keeps them in COMMON
 * /omp_dot/, include/openmp.fi).
 * ====================================================================== */
static double omp_dot1, omp_dot2, omp_dot3, omp_dot4;

static double dot_ompL4(const double *a, const double *b, int32_t n) {
  /* Matvec_omp.f:1247-1296 */
  int32_t resto = n % 4;
#pragma omp single
  {
    omp_dot2 = 0.0;
    omp_dot3 = 0.0;
    omp_dot4 = 0.0;
    if (resto == 0)
      omp_dot1 = 0.0;
    else if (resto == 1)
      omp_dot1 = F1(a, 1) * F1(b, 1);
    else if (resto == 2)
      omp_dot1 = F1(a, 1) * F1(b, 1) + F1(a, 2) * F1(b, 2);
    else
      omp_dot1 = F1(a, 1) * F1(b, 1) + F1(a, 2) * F1(b, 2) + F1(a, 3) * F1(b, 3);
  }
#pragma omp for schedule(static) reduction(+ : omp_dot1, omp_dot2, omp_dot3, omp_dot4)
  for (int32_t i = 1 + resto; i <= n; i += 4) {
    omp_dot1 = omp_dot1 + F1(a, i) * F1(b, i);
    omp_dot2 = omp_dot2 + F1(a, i + 1) * F1(b, i + 1);
    omp_dot3 = omp_dot3 + F1(a, i + 2) * F1(b, i + 2);
    omp_dot4 = omp_dot4 + F1(a, i + 3) * F1(b, i + 3);
  }
  double d = omp_dot1 + omp_dot2 + omp_dot3 + omp_dot4;
#pragma omp barrier
  return d;
}

static void matvec_csrd_omp(const double *ad, const double *a, const double *dum,
                            const double *x, double *y, const int32_t *ia,
                            const int32_t *ja, int32_t neq) {
  /* Matvec_omp.f:21-53 (and the ilu2 variant :76-120, which sums in the
   * same order) */
  (void)dum;
#pragma omp for schedule(static)
  for (int32_t i = 1; i <= neq; ++i) {
    double t = F1(ad, i) * F1(x, i);
    for (int32_t j = F1(ia, i); j <= F1(ia, i + 1) - 1; ++j)
      t = t + F1(a, j) * F1(x, F1(ja, j));
    F1(y, i) = t;
  }
}

static void matvec_ellpack_omp(const double *ad, const double *a,
                               const double *dum, const double *x, double *y,
                               const int32_t *nl, const int32_t *ja,
                               int32_t neq) {
  /* Matvec_omp.f:1036-1086 */
  (void)dum;
  int32_t w = F1(nl, 1);
  if (w == 3) {
#pragma omp for schedule(static)
    for (int32_t i = 1; i <= neq; ++i) {
      double t4 = F1(ad, i) * F1(x, i);
      double t1 = F2(a, 3, 1, i) * F1(x, F2(ja, 3, 1, i));
      double t2 = F2(a, 3, 2, i) * F1(x, F2(ja, 3, 2, i));
      double t3 = F2(a, 3, 3, i) * F1(x, F2(ja, 3, 3, i));
      F1(y, i) = t1 + t2 + t3 + t4;
    }
  } else if (w == 4) {
#pragma omp for schedule(static)
    for (int32_t i = 1; i <= neq; ++i) {
      double t5 = F1(ad, i) * F1(x, i);
      double t1 = F2(a, 4, 1, i) * F1(x, F2(ja, 4, 1, i));
      double t2 = F2(a, 4, 2, i) * F1(x, F2(ja, 4, 2, i));
      double t3 = F2(a, 4, 3, i) * F1(x, F2(ja, 4, 3, i));
      double t4 = F2(a, 4, 4, i) * F1(x, F2(ja, 4, 4, i));
      F1(y, i) = t1 + t2 + t3 + t4 + t5;
    }
  }
}

/* Symmetric CSRD (strict lower part stored) with per-thread buffers:
 * Matvec_omp.f:310-372, partition from Matrix_partition.f:26-184. */
#define OREF_MAXT 256
static int32_t thr_begin[OREF_MAXT + 1], thr_end[OREF_MAXT + 1],
    thr_height[OREF_MAXT + 1];
static int32_t sym_nthreads;

static int32_t partition_matrix(const int32_t *ia, const int32_t *ja,
                                int32_t neq, int32_t nth) {
  /* partition_csrc_bynonzeros, Matrix_partition.f:78-107.  The reference
   * loop can walk past neq when rows are short; the guard line <= neq is
   * an addition. */
  int32_t nad = F1(ia, neq + 1) - 1;
  int32_t mean_variables = (2 * nad + neq) / nth + 1;
  int32_t line = 2;
  thr_begin[1] = 1;
  for (int32_t i = 1; i <= nth - 1; ++i) {
    int32_t size = 0;
    thr_end[i] = 0;
    while (line <= neq + 1) {
      int32_t tam = 2 * (F1(ia, line) - F1(ia, line - 1)) + 1;
      if (size + tam > mean_variables) break;
      size += tam;
      thr_end[i] = line - 1;
      thr_begin[i + 1] = line;
      line++;
    }
  }
  thr_end[nth] = neq;
  /* compute_effective_work, Matrix_partition.f:168-184 */
  for (int32_t t = 1; t <= nth; ++t) {
    int32_t h = thr_begin[t];
    for (int32_t i = thr_begin[t]; i <= thr_end[t]; ++i)
      for (int32_t k = F1(ia, i); k <= F1(ia, i + 1) - 1; ++k)
        if (F1(ja, k) < h) h = F1(ja, k);
    thr_height[t] = h;
  }
  for (int32_t t = 1; t <= nth; ++t)
    if (thr_height[t] <= 0 || thr_begin[t] <= 0 || thr_end[t] <= 0) return -1;
  return 0;
}

static double *sym_thread_y;

static void matvec_csrd_sym_omp(const double *ad, const double *dum,
                                const double *al, const double *x, double *y,
                                const int32_t *ia, const int32_t *ja,
                                int32_t neq) {
  (void)dum;
  double *thread_y = sym_thread_y;
  int32_t tid = 1;
#ifdef _OPENMP
  tid = omp_get_thread_num() + 1;
#endif
  for (int32_t i = 1; i <= sym_nthreads; ++i) {
    size_t inc = (size_t)(i - 1) * neq;
#pragma omp for schedule(static)
    for (int32_t j = thr_height[i]; j <= thr_begin[i] - 1; ++j)
      thread_y[inc + j - 1] = 0.0;
  }
  size_t inc = (size_t)(tid - 1) * neq;
#pragma omp barrier
  for (int32_t i = thr_begin[tid]; i <= thr_end[tid]; ++i) {
    F1(y, i) = 0.0;
    double xi = F1(x, i);
    double t = F1(ad, i) * xi;
    for (int32_t k = F1(ia, i); k <= F1(ia, i + 1) - 1; ++k) {
      int32_t jak = F1(ja, k);
      double s = F1(al, k);
      t = t + s * F1(x, jak);
      thread_y[inc + jak - 1] = thread_y[inc + jak - 1] + s * xi;
    }
    thread_y[inc + i - 1] = t;
  }
#pragma omp barrier
  for (int32_t i = 1; i <= sym_nthreads; ++i) {
    size_t inc2 = (size_t)(i - 1) * neq;
#pragma omp for schedule(static)
    for (int32_t j = thr_height[i]; j <= thr_end[i]; ++j)
      F1(y, j) = F1(y, j) + thread_y[inc2 + j - 1];
  }
}

static int32_t pcg_omp(int32_t neq, const int32_t *ia, const int32_t *ja,
                       const double *ad, const double *au, const double *al,
                       const double *m, double *b, double *x, double *z,
                       double *r, double tol, int32_t maxit, matvec_fn matvec,
                       int32_t init, int32_t nthreads, int32_t stop_rule,
                       oref_stats *st) {
  /* Iterativos_omp.f:30-127.  stop_rule 0 is the reference's test
   * sqrt|r.z| < tol sqrt|r0.z0| (:57,:88).  stop_rule 1 (not in the
   * reference) stops on ||r||2 < tol ||b||2 instead, the rule the GPU
   * solves use with fvc_opts.stop_rule = 1; it adds one dot_ompL4(r, r)
   * per iteration and changes nothing else. */
  int32_t status = OREF_OK, jout = 0;
  double energy = 0.0, dout = 0.0, convout = 0.0;
#pragma omp parallel num_threads(nthreads)
  {
    double d, conv, alpha, beta, crit = 0.0, bnorm = 0.0;
    int32_t i, j;
    if (init) {
#pragma omp for schedule(static)
      for (i = 1; i <= neq; ++i) F1(x, i) = 0.0;
    }
    if (stop_rule == 1) bnorm = sqrt(dot_ompL4(b, b, neq));
    matvec(ad, au, al, x, z, ia, ja, neq);
#pragma omp for schedule(static)
    for (i = 1; i <= neq; ++i) {
      F1(r, i) = F1(b, i) - F1(z, i);
      F1(z, i) = F1(r, i) / F1(m, i);
      F1(b, i) = F1(z, i);
    }
    d = dot_ompL4(r, z, neq);
    conv = (stop_rule == 1) ? tol * bnorm : tol * sqrt(fabs(d));
    for (j = 1; j <= maxit; ++j) {
      matvec(ad, au, al, b, z, ia, ja, neq);
      alpha = d / dot_ompL4(b, z, neq);
#pragma omp for schedule(static)
      for (i = 1; i <= neq; ++i) {
        F1(x, i) = F1(x, i) + alpha * F1(b, i);
        F1(r, i) = F1(r, i) - alpha * F1(z, i);
        F1(z, i) = F1(r, i) / F1(m, i);
      }
      beta = dot_ompL4(r, z, neq) / d;
#pragma omp for schedule(static)
      for (i = 1; i <= neq; ++i) F1(b, i) = F1(z, i) + beta * F1(b, i);
      d = beta * d;
      crit = (stop_rule == 1) ? sqrt(dot_ompL4(r, r, neq)) : sqrt(fabs(d));
      if (crit < conv) break;
    }
    double en = 0.0;
    if (j <= maxit) {
      matvec(ad, au, al, x, z, ia, ja, neq);
      en = dot_ompL4(x, z, neq);
    }
#pragma omp single
    {
      jout = j;
      dout = crit;
      convout = conv;
      energy = en;
      if (j > maxit) status = OREF_NOCONV;
    }
  }
  st->iterations = (jout > maxit) ? maxit : jout;
  st->energy = energy;
  st->conv = convout;
  st->final_crit = dout;
  st->status = status;
  return status;
}

static int32_t pbicgstab_omp(int32_t neq, const int32_t *ia, const int32_t *ja,
                             const double *ad, const double *au,
                             const double *al, const double *m, double *b,
                             double *x, double *t, double *v, double *r,
                             double *p, double *z, double tol, int32_t maxit,
                             matvec_fn matvec, int32_t init, int32_t nthreads,
                             oref_stats *st) {
  /* Iterativos_omp.f:161-274 */
  int32_t status = OREF_OK, jout = 0;
  double energy = 0.0, bout = 0.0, convout = 0.0;
#pragma omp parallel num_threads(nthreads)
  {
    double d, conv, alpha, beta = 0.0, rr0, w;
    int32_t i, j;
    if (init) {
#pragma omp for schedule(static)
      for (i = 1; i <= neq; ++i) F1(x, i) = 0.0;
    }
    matvec(ad, au, al, x, z, ia, ja, neq);
#pragma omp for schedule(static)
    for (i = 1; i <= neq; ++i) {
      F1(r, i) = F1(b, i) - F1(z, i);
      F1(p, i) = F1(r, i);
      F1(b, i) = F1(p, i);
      F1(z, i) = F1(p, i) / F1(m, i);
    }
    d = dot_ompL4(r, z, neq);
    conv = tol * sqrt(fabs(d));
    for (j = 1; j <= maxit; ++j) {
      matvec(ad, au, al, z, v, ia, ja, neq);
      rr0 = dot_ompL4(b, r, neq);
      alpha = rr0 / dot_ompL4(v, r, neq);
#pragma omp for schedule(static)
      for (i = 1; i <= neq; ++i) {
        F1(x, i) = F1(x, i) + alpha * F1(z, i);
        F1(b, i) = F1(b, i) - alpha * F1(v, i);
        F1(z, i) = F1(b, i) / F1(m, i);
      }
      matvec(ad, au, al, z, t, ia, ja, neq);
      double tb = dot_ompL4(t, b, neq);
      w = tb / dot_ompL4(t, t, neq);
#pragma omp for schedule(static)
      for (i = 1; i <= neq; ++i) {
        F1(x, i) = F1(x, i) + w * F1(z, i);
        F1(b, i) = F1(b, i) - w * F1(t, i);
      }
      beta = dot_ompL4(b, z, neq) / d;
      if (sqrt(fabs(beta)) < conv) break;
      beta = (dot_ompL4(r, b, neq) / rr0) * (alpha / w);
#pragma omp for schedule(static)
      for (i = 1; i <= neq; ++i) {
        F1(p, i) = F1(b, i) + beta * (F1(p, i) - w * F1(v, i));
        F1(z, i) = F1(p, i) / F1(m, i);
      }
    }
    double en = 0.0;
    if (j <= maxit) {
      matvec(ad, au, al, x, z, ia, ja, neq);
      en = dot_ompL4(x, z, neq);
    }
#pragma omp single
    {
      jout = j;
      bout = beta;
      convout = conv;
      energy = en;
      if (j > maxit) status = OREF_NOCONV;
    }
  }
  st->iterations = (jout > maxit) ? maxit : jout;
  st->energy = energy;
  st->conv = convout;
  st->final_crit = sqrt(fabs(bout));
  st->status = status;
  return status;
}

/* ======================================================================
 * Solver.f:28-346 dispatch
 * ====================================================================== */
static void wrap_matvec_csrd(const double *ad, const double *au, const double *al,
                             const double *x, double *y, const int32_t *ia,
                             const int32_t *ja, int32_t neq) {
  oref_matvec_csrd(ad, au, al, x, y, ia, ja, neq);
}

int32_t oref_solver(double *ad, double *au, double *al, double *x, double *b,
                    const int32_t *iax, const int32_t *ja, int32_t neq,
                    int32_t nad, int32_t unsym, double tol, int32_t maxit,
                    int32_t code, int32_t matriz, int32_t omp_threads,
                    oref_stats *st) {
  (void)nad;
  const int32_t k = 15;
  int32_t openmp = omp_threads > 0;
  int32_t status = OREF_UNSUPPORTED;
  memset(st, 0, sizeof(*st));
  st->status = OREF_UNSUPPORTED;
  if (openmp && !unsym) {
    if (omp_threads > OREF_MAXT) return OREF_UNSUPPORTED;
    sym_nthreads = omp_threads;
    if (matriz == 1 && partition_matrix(iax, ja, neq, omp_threads) != 0)
      return OREF_UNSUPPORTED;
    sym_thread_y = (double *)calloc((size_t)omp_threads * neq, sizeof(double));
  }
  if (code == 1) {
    double *r = (double *)calloc((size_t)neq, sizeof(double));
    double *z = (double *)calloc((size_t)neq, sizeof(double));
    double *m = (double *)calloc((size_t)neq, sizeof(double));
    /* Solver.f:84 m = ad.  For matriz 2 (diagonal inside the CSR values)
     * the reference copies the first neq values, which is not the
     * diagonal; the diagonal (the entry whose column is the row) is used
     * here instead. */
    if (matriz == 2) {
      for (int32_t i = 1; i <= neq; ++i)
        for (int32_t kk = F1(iax, i); kk < F1(iax, i + 1); ++kk)
          if (F1(ja, kk) == i) F1(m, i) = F1(ad, kk);
    } else {
      memcpy(m, ad, sizeof(double) * (size_t)neq);
    }
    if (matriz == 1) {
      if (openmp) {
        if (unsym)
          status = pcg_omp(neq, iax, ja, ad, au, al, m, b, x, z, r, tol, maxit,
                           matvec_csrd_omp, 0, omp_threads, 0, st);
        else
          status = pcg_omp(neq, iax, ja, ad, au, al, m, b, x, z, r, tol, maxit,
                           matvec_csrd_sym_omp, 0, omp_threads, 0, st);
      } else {
        if (unsym)
          status = pcg(neq, iax, ja, ad, au, al, m, b, x, z, r, tol, maxit,
                       wrap_matvec_csrd, 1, st);
        else
          status = pcg(neq, iax, ja, ad, au, al, m, b, x, z, r, tol, maxit,
                       oref_matvec_csrd_sym, 1, st);
      }
    } else if (matriz == 2) {
      /* Solver.f:142-143 passes no dot routine (reference bug); the
       * evident intent, PCG with matvec_csr, is restated. */
      status = pcg(neq, iax, ja, ad, au, al, m, b, x, z, r, tol, maxit,
                   oref_matvec_csr, 1, st);
    } else if (matriz == 3) {
      /* Solver.f:148-149, same missing-dot bug; intent restated. */
      status = pcg(neq, iax, ja, ad, au, al, m, b, x, z, r, tol, maxit,
                   oref_matvec_csrc_sym, 1, st);
    } else if (matriz == 4) {
      if (openmp)
        status = pcg_omp(neq, iax, ja, ad, au, al, m, b, x, z, r, tol, maxit,
                         matvec_ellpack_omp, 0, omp_threads, 0, st);
      else
        status = pcg(neq, iax, ja, ad, au, al, m, b, x, z, r, tol, maxit,
                     oref_matvec_ellpack, 0, st);
    }
    free(r);
    free(z);
    free(m);
  } else if (code == 2) {
    double *r = (double *)calloc((size_t)neq, sizeof(double));
    double *z = (double *)calloc((size_t)neq, sizeof(double));
    double *m = (double *)calloc((size_t)neq, sizeof(double));
    double *t = (double *)calloc((size_t)neq, sizeof(double));
    double *v = (double *)calloc((size_t)neq, sizeof(double));
    double *p = (double *)calloc((size_t)neq, sizeof(double));
    memcpy(m, ad, sizeof(double) * (size_t)neq);
    if (matriz == 1) {
      if (unsym) {
        if (openmp)
          status = pbicgstab_omp(neq, iax, ja, ad, au, al, m, b, x, t, v, r, p,
                                 z, tol, maxit, matvec_csrd_omp, 1, omp_threads,
                                 st);
        else
          status = pbicgstab(neq, iax, ja, ad, au, al, m, b, x, t, v, r, p, z,
                             tol, maxit, wrap_matvec_csrd, 1, st);
      } else {
        status = pbicgstab(neq, iax, ja, ad, au, al, m, b, x, t, v, r, p, z,
                           tol, maxit, oref_matvec_csrd_sym, 1, st);
      }
    } else if (matriz == 3) {
      if (unsym)
        status = pbicgstab(neq, iax, ja, ad, au, al, m, b, x, t, v, r, p, z,
                           tol, maxit, oref_matvec_csrc, 1, st);
      else
        status = pbicgstab(neq, iax, ja, ad, au, al, m, b, x, t, v, r, p, z,
                           tol, maxit, oref_matvec_csrc_sym, 1, st);
    } else if (matriz == 4) {
      if (openmp)
        status = pbicgstab_omp(neq, iax, ja, ad, au, al, m, b, x, t, v, r, p, z,
                               tol, maxit, matvec_ellpack_omp, 0, omp_threads,
                               st);
      else
        status = pbicgstab(neq, iax, ja, ad, au, al, m, b, x, t, v, r, p, z,
                           tol, maxit, oref_matvec_ellpack, 0, st);
    } else {
      status = OREF_UNSUPPORTED; /* Solver.f:224-227 */
      st->status = status;
    }
    free(r);
    free(z);
    free(m);
    free(t);
    free(v);
    free(p);
  } else if (code == 3) {
    double *g = (double *)calloc((size_t)(k + 1) * neq, sizeof(double));
    double *h = (double *)calloc((size_t)(k + 1) * k, sizeof(double));
    double *m = (double *)calloc((size_t)neq, sizeof(double));
    double *y = (double *)calloc((size_t)k, sizeof(double));
    double *c = (double *)calloc((size_t)k, sizeof(double));
    double *s = (double *)calloc((size_t)k, sizeof(double));
    double *e = (double *)calloc((size_t)k + 1, sizeof(double));
    memcpy(m, ad, sizeof(double) * (size_t)neq);
    matvec_fn mv = NULL;
    if (matriz == 1)
      mv = unsym ? wrap_matvec_csrd : oref_matvec_csrd_sym;
    else if (matriz == 3)
      mv = unsym ? oref_matvec_csrc : oref_matvec_csrc_sym;
    if (mv)
      status = gmres(neq, iax, ja, ad, au, al, m, b, x, k, g, h, y, c, s, e,
                     tol, maxit, mv, st);
    else
      st->status = status = OREF_UNSUPPORTED; /* Solver.f:305-308 */
    free(g);
    free(h);
    free(m);
    free(y);
    free(c);
    free(s);
    free(e);
  }
  if (sym_thread_y) {
    free(sym_thread_y);
    sym_thread_y = NULL;
  }
  return status;
}

int32_t oref_pcg_omp_sample(double *ad, double *au, double *al, double *x,
                            double *b, const int32_t *iax, const int32_t *ja,
                            int32_t neq, int32_t nad, double tol, int32_t maxit,
                            int32_t matriz, int32_t nthreads, int32_t init,
                            int32_t stop_rule, oref_stats *st) {
  (void)nad;
  memset(st, 0, sizeof(*st));
  double *r = (double *)calloc((size_t)neq, sizeof(double));
  double *z = (double *)calloc((size_t)neq, sizeof(double));
  double *m = (double *)malloc(sizeof(double) * (size_t)neq);
  memcpy(m, ad, sizeof(double) * (size_t)neq);
  int32_t status;
  if (matriz == 4)
    status = pcg_omp(neq, iax, ja, ad, au, al, m, b, x, z, r, tol, maxit,
                     matvec_ellpack_omp, init, nthreads, stop_rule, st);
  else
    status = pcg_omp(neq, iax, ja, ad, au, al, m, b, x, z, r, tol, maxit,
                     matvec_csrd_omp, init, nthreads, stop_rule, st);
  free(r);
  free(z);
  free(m);
  return status;
}

/* ======================================================================
 * Pressure-correction assembly: src/Pform.f:277-432 (cell loop, gather),
 * src/Celllib.f:695-794 (cellGeom2D), src/Celllib.f:596-655 (vectorKm2d),
 * src/CellibPressure.f:476-572 (cell_si_p_i_ggl, iws = 1, matrix part),
 * src/Assbly.f:32-54.  Boundary faces are walls (pedge 0: a = 0); the
 * optional pin_cell carries pedge(idCell) = -1 (the 1e60 pin, :557).
 * Generalised to mixed meshes by using each cell's own vertex count
 * (the reference has one element type per mesh).
 * ====================================================================== */
static int32_t cell_nsides(const int32_t *ix, int32_t ld, int32_t c, int32_t nshared) {
  int32_t s = 0;
  while (s < nshared && s < ld && ix[(size_t)(c - 1) * ld + s] > 0) s++;
  return s;
}

void oref_pform_pressure(const double *coor, int32_t nnode, const int32_t *ix, int32_t ld,
                         int32_t numel, int32_t nshared, const int32_t *nelcon,
                         const int32_t *num, const double *kprop, const double *dsim,
                         int32_t pin_cell, int32_t int_vel, int32_t matriz, int32_t unsym,
                         const int32_t *ia, const int32_t *ja, double *ad, double *au) {
  (void)nnode;
  enum { MS = 4 };
  const int32_t idcell = nshared + 1;
  for (int32_t nel = 1; nel <= numel; ++nel) {
    /* gather: x(2, MS, nshared+1), nsides per local cell */
    double x[2][MS][MS + 1];
    int32_t nsl[MS + 1], viz[MS], ld_[MS + 1];
    double kk[MS + 1], dd[2][MS + 1];
    for (int32_t i = 1; i <= idcell; ++i) ld_[i - 1] = 0;
    for (int32_t j = 1; j <= nshared; ++j) {
      int32_t v = F2(nelcon, nshared, j, nel);
      viz[j - 1] = v;
      if (v > 0) {
        ld_[j - 1] = F1(num, v);
        nsl[j - 1] = cell_nsides(ix, ld, v, nshared);
        kk[j - 1] = F1(kprop, v);
        dd[0][j - 1] = F2(dsim, 2, 1, v);
        dd[1][j - 1] = F2(dsim, 2, 2, v);
        for (int32_t i = 1; i <= nsl[j - 1]; ++i) {
          int32_t no = F2(ix, ld, i, v);
          x[0][i - 1][j - 1] = F2(coor, 2, 1, no);
          x[1][i - 1][j - 1] = F2(coor, 2, 2, no);
        }
      }
    }
    ld_[idcell - 1] = F1(num, nel);
    nsl[idcell - 1] = cell_nsides(ix, ld, nel, nshared);
    kk[idcell - 1] = F1(kprop, nel);
    dd[0][idcell - 1] = F2(dsim, 2, 1, nel);
    dd[1][idcell - 1] = F2(dsim, 2, 2, nel);
    for (int32_t i = 1; i <= nsl[idcell - 1]; ++i) {
      int32_t no = F2(ix, ld, i, nel);
      x[0][i - 1][idcell - 1] = F2(coor, 2, 1, no);
      x[1][i - 1][idcell - 1] = F2(coor, 2, 2, no);
    }
    const int32_t ns = nsl[idcell - 1];
    /* cellGeom2D */
    double xc[2][MS + 1], mksi[MS], meta[MS], ksi[2][MS], eta[2][MS], n[2][MS], xm[2][MS], ca[MS];
    for (int32_t i = 1; i <= idcell; ++i) {
      if (i <= nshared && viz[i - 1] <= 0) continue;
      for (int32_t j = 1; j <= 2; ++j) {
        double s = 0.0;
        for (int32_t l = 1; l <= nsl[i - 1]; ++l) s = s + x[j - 1][l - 1][i - 1];
        xc[j - 1][i - 1] = (1.0 / nsl[i - 1]) * s;
      }
    }
    for (int32_t l = 1; l <= ns; ++l) {
      int32_t l2 = (l % ns) + 1;
      eta[0][l - 1] = x[0][l2 - 1][idcell - 1] - x[0][l - 1][idcell - 1];
      eta[1][l - 1] = x[1][l2 - 1][idcell - 1] - x[1][l - 1][idcell - 1];
    }
    for (int32_t i = 1; i <= ns; ++i) {
      mksi[i - 1] = 0.0;
      if (viz[i - 1] > 0) {
        for (int32_t j = 1; j <= 2; ++j) {
          ksi[j - 1][i - 1] = xc[j - 1][i - 1] - xc[j - 1][idcell - 1];
          mksi[i - 1] = ksi[j - 1][i - 1] * ksi[j - 1][i - 1] + mksi[i - 1];
        }
        mksi[i - 1] = sqrt(mksi[i - 1]);
      }
      meta[i - 1] = 0.0;
      for (int32_t j = 1; j <= 2; ++j) meta[i - 1] = meta[i - 1] + eta[j - 1][i - 1] * eta[j - 1][i - 1];
      meta[i - 1] = sqrt(meta[i - 1]);
    }
    for (int32_t j = 1; j <= 2; ++j)
      for (int32_t i = 1; i <= ns; ++i) {
        eta[j - 1][i - 1] = eta[j - 1][i - 1] / meta[i - 1];
        if (viz[i - 1] > 0) ksi[j - 1][i - 1] = ksi[j - 1][i - 1] / mksi[i - 1];
      }
    for (int32_t l = 1; l <= ns; ++l) {
      n[0][l - 1] = eta[1][l - 1];
      n[1][l - 1] = -eta[0][l - 1];
    }
    for (int32_t i = 1; i <= ns; ++i) {
      int32_t i2 = (i % ns) + 1;
      xm[0][i - 1] = 0.5 * (x[0][i2 - 1][idcell - 1] + x[0][i - 1][idcell - 1]);
      xm[1][i - 1] = 0.5 * (x[1][i2 - 1][idcell - 1] + x[1][i - 1][idcell - 1]);
      ca[i - 1] = (xm[0][i - 1] - xc[0][idcell - 1]) * n[0][i - 1] +
                  (xm[1][i - 1] - xc[1][idcell - 1]) * n[1][i - 1];
    }
    /* vectorKm2d: ghost centroids for boundary faces, then mKsiF */
    double xcg[2][MS], mksif[MS];
    for (int32_t i = 1; i <= ns; ++i) {
      if (viz[i - 1] < 0) {
        for (int32_t j = 1; j <= 2; ++j)
          xcg[j - 1][i - 1] = xc[j - 1][idcell - 1] + 2.0 * ca[i - 1] * n[j - 1][i - 1];
      } else {
        for (int32_t j = 1; j <= 2; ++j) xcg[j - 1][i - 1] = xc[j - 1][i - 1];
      }
    }
    for (int32_t i = 1; i <= ns; ++i) {
      int32_t no1 = i, no2 = (i % ns) + 1;
      double a1 = xcg[1][i - 1] - xc[1][idcell - 1];
      double b1 = xc[0][idcell - 1] - xcg[0][i - 1];
      double c1 = xcg[0][i - 1] * xc[1][idcell - 1] - xc[0][idcell - 1] * xcg[1][i - 1];
      double a2 = x[1][no1 - 1][idcell - 1] - x[1][no2 - 1][idcell - 1];
      double b2 = x[0][no2 - 1][idcell - 1] - x[0][no1 - 1][idcell - 1];
      double c2 = x[0][no1 - 1][idcell - 1] * x[1][no2 - 1][idcell - 1] -
                  x[0][no2 - 1][idcell - 1] * x[1][no1 - 1][idcell - 1];
      double det = a1 * b2 - a2 * b1;
      double m11 = (1.0 / det) * b2, m12 = -(1.0 / det) * b1;
      double m21 = -(1.0 / det) * a2, m22 = (1.0 / det) * a1;
      double f1 = -c1, f2 = -c2;
      double xi1 = m11 * f1 + m12 * f2, xi2 = m21 * f1 + m22 * f2;
      double kf1 = xi1 - xc[0][idcell - 1], kf2 = xi2 - xc[1][idcell - 1];
      mksif[i - 1] = sqrt(kf1 * kf1 + kf2 * kf2);
    }
    /* cell_si_p_i_ggl iws = 1, matrix part */
    double la[MS + 1];
    double sp = 0.0;
    for (int32_t i = 1; i <= nshared; ++i) la[i - 1] = 0.0;
    for (int32_t i = 1; i <= ns; ++i) {
      if (viz[i - 1] < 0) {
        la[i - 1] = 0.0;
        continue;
      }
      double alpha = mksif[i - 1] / mksi[i - 1];
      double kf, ndd;
      double ddf1 = (1.0 - alpha) * dd[0][idcell - 1] + alpha * dd[0][i - 1];
      double ddf2 = (1.0 - alpha) * dd[1][idcell - 1] + alpha * dd[1][i - 1];
      if (int_vel == 5) {
        kf = (1.0 - alpha) * kk[idcell - 1] + alpha * kk[i - 1];
        ndd = 0.5 * (ddf1 + ddf2);
      } else {
        kf = kk[idcell - 1];
        double d1 = ddf1 * n[0][i - 1], d2 = ddf2 * n[1][i - 1];
        ndd = d1 * n[0][i - 1] + d2 * n[1][i - 1];
      }
      double nk = n[0][i - 1] * ksi[0][i - 1] + n[1][i - 1] * ksi[1][i - 1];
      la[i - 1] = (kf * meta[i - 1] * ndd) / (nk * mksi[i - 1]);
    }
    if (pin_cell == nel) sp = sp + 1.0e60;
    la[idcell - 1] = sp;
    for (int32_t i = 1; i <= nshared; ++i) la[idcell - 1] = la[idcell - 1] + la[i - 1];
    oref_assbly(ad, au, au, NULL, ia, ja, la, 0.0, ld_, nshared, matriz, unsym, 0, 1);
  }
}
