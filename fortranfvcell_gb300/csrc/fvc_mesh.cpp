// fvc_mesh.cpp -- host-side mesh -> equation-graph tools of libfvcgpu.
//
// Integer setup work done once per mesh: face adjacency, reverse
// Cuthill-McKee ordering, equation numbering and the sparse index
// structures.  The outputs are the reference's arrays, value for value
// (1-based), so a Fortran caller can hand them straight to fvc_solver:
//   adjacency   : src/Adjacency.f:1-189 (result; computed by edge matching)
//   RCM         : src/Reord.f:6-468     (same SPARSPAK steps and tie rules)
//   numbering   : src/Numeq.f:4-25
//   structures  : src/Datastruct.f:27-179, src/Csr.f:21-110,
//                 src/Graph.f:45-93, src/EllPack.f:19-42
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/fvcgpu.h"

namespace {

// Number of sides of cell c: its leading nonzero node slots.
inline int cell_sides(const int32_t *ix, int ld, int c, int nshared) {
  int s = 0;
  while (s < nshared && s < ld && ix[(size_t)c * ld + s] > 0) ++s;
  return s;
}

// Cell graph in 0-based adjacency-list form, neighbours in side order
// (the order src/Graph.f:18-41 conv_graph produces).
struct CellGraph {
  std::vector<int> start;  // n+1
  std::vector<int> nbr;
};

CellGraph graph_from_nelcon(const int32_t *nelcon, int numel, int nshared) {
  CellGraph g;
  g.start.assign((size_t)numel + 1, 0);
  g.nbr.reserve((size_t)numel * nshared);
  for (int c = 0; c < numel; ++c) {
    for (int s = 0; s < nshared; ++s) {
      int v = nelcon[(size_t)c * nshared + s];
      if (v != -1) g.nbr.push_back(v - 1);
    }
    g.start[c + 1] = (int)g.nbr.size();
  }
  return g;
}

// Reverse Cuthill-McKee over one graph.  The routine boundaries follow
// SPARSPAK (rootls / fnroot / degree / rcm) because the reference's
// permutation depends on their exact visiting and tie rules.
class Rcm {
 public:
  explicit Rcm(const CellGraph &g)
      : g_(g), n_((int)g.start.size() - 1), free_(n_, 1), deg_(n_, 0),
        levels_(n_ + 1, 0), seen_(n_, 0) {}

  // order[k] = cell placed at position k (0-based)
  std::vector<int> run() {
    std::vector<int> order;
    order.reserve(n_);
    std::vector<int> ls;
    for (int i = 0; i < n_; ++i) {
      if (!free_[i]) continue;
      int root = i;
      int nlvl = 0;
      pseudo_peripheral(root, nlvl, ls);
      size_t first = order.size();
      cuthill_mckee(root, order);
      std::reverse(order.begin() + first, order.end());
      if ((int)order.size() >= n_) break;
    }
    return order;
  }

 private:
  // Level structure rooted at root over the free nodes (Reord.f:294-357).
  // Returns the component size; levels_[0..nlvl] holds level starts.
  int level_structure(int root, int &nlvl, std::vector<int> &ls) {
    ls.clear();
    ls.push_back(root);
    free_[root] = 0;
    nlvl = 0;
    size_t lo = 0;
    while (lo < ls.size()) {
      size_t hi = ls.size();
      levels_[nlvl++] = (int)lo;
      for (size_t q = lo; q < hi; ++q) {
        int v = ls[q];
        for (int k = g_.start[v]; k < g_.start[v + 1]; ++k) {
          int w = g_.nbr[k];
          if (free_[w]) {
            free_[w] = 0;
            ls.push_back(w);
          }
        }
      }
      lo = hi;
    }
    levels_[nlvl] = (int)ls.size();
    for (int v : ls) free_[v] = 1;
    return (int)ls.size();
  }

  // Gibbs-Poole-Stockmeyer style root search (Reord.f:112-164).  The last
  // level is scanned keeping the LAST node whose free degree is >= the
  // running value (the reference compares with .ge.).
  void pseudo_peripheral(int &root, int &nlvl, std::vector<int> &ls) {
    int csize = level_structure(root, nlvl, ls);
    if (nlvl == 1 || nlvl == csize) return;
    for (;;) {
      int first = levels_[nlvl - 1];
      int best = csize;
      root = ls[first];
      if (first + 1 != csize) {
        for (int q = first; q < csize; ++q) {
          int v = ls[q];
          int d = 0;
          for (int k = g_.start[v]; k < g_.start[v + 1]; ++k)
            if (free_[g_.nbr[k]]) ++d;
          if (d >= best) {
            root = v;
            best = d;
          }
        }
      }
      int nnew = 0;
      level_structure(root, nnew, ls);
      if (nnew <= nlvl) return;
      nlvl = nnew;
      if (nlvl >= csize) return;
    }
  }

  // Degrees of the free nodes of root's component, counted over free
  // neighbours (Reord.f:358-457).
  void degrees(int root, std::vector<int> &comp) {
    comp.clear();
    comp.push_back(root);
    seen_[root] = 1;
    for (size_t q = 0; q < comp.size(); ++q) {
      int v = comp[q];
      int d = 0;
      for (int k = g_.start[v]; k < g_.start[v + 1]; ++k) {
        int w = g_.nbr[k];
        if (!free_[w]) continue;
        ++d;
        if (!seen_[w]) {
          seen_[w] = 1;
          comp.push_back(w);
        }
      }
      deg_[v] = d;
    }
    for (int v : comp) seen_[v] = 0;
  }

  // Cuthill-McKee numbering of root's component appended to order
  // (Reord.f:165-293, before the reversal): each node's newly numbered
  // neighbours are ordered by increasing degree, ties kept in visit order.
  void cuthill_mckee(int root, std::vector<int> &order) {
    std::vector<int> comp;
    degrees(root, comp);
    size_t base = order.size();
    order.push_back(root);
    free_[root] = 0;
    if (comp.size() <= 1) return;
    size_t head = base;
    while (head < order.size()) {
      int v = order[head++];
      size_t fresh = order.size();
      for (int k = g_.start[v]; k < g_.start[v + 1]; ++k) {
        int w = g_.nbr[k];
        if (free_[w]) {
          free_[w] = 0;
          order.push_back(w);
        }
      }
      std::stable_sort(order.begin() + fresh, order.end(),
                       [this](int a, int b) { return deg_[a] < deg_[b]; });
    }
  }

  const CellGraph &g_;
  int n_;
  std::vector<char> free_;
  std::vector<int> deg_;
  std::vector<int> levels_;
  std::vector<char> seen_;
};

}  // namespace

extern "C" {

int32_t fvc_mesh_adjacency(const int32_t *ix, int32_t ld, int32_t nnode,
                           int32_t numel, int32_t nshared, int32_t *nelcon) {
  if (!ix || !nelcon || ld < 3 || nnode <= 0 || numel <= 0 || nshared < 3)
    return FVC_ERR_ARG;
  // Directed edges grouped by their start node (counting sort), then each
  // edge a->b looks for the twin b->a among the edges leaving b.
  std::vector<int> cnt((size_t)nnode + 1, 0);
  for (int c = 0; c < numel; ++c) {
    int ns = cell_sides(ix, ld, c, nshared);
    if (ns < 3) return FVC_ERR_ARG;
    for (int s = 0; s < ns; ++s) {
      int a = ix[(size_t)c * ld + s];
      if (a < 1 || a > nnode) return FVC_ERR_ARG;
      cnt[a]++;
    }
  }
  std::vector<int> off((size_t)nnode + 2, 0);
  for (int v = 1; v <= nnode; ++v) off[v + 1] = off[v] + cnt[v];
  std::vector<int> fill(off.begin(), off.end());
  std::vector<int> edge_cell(off[nnode + 1]), edge_side(off[nnode + 1]),
      edge_end(off[nnode + 1]);
  for (int c = 0; c < numel; ++c) {
    int ns = cell_sides(ix, ld, c, nshared);
    for (int s = 0; s < ns; ++s) {
      int a = ix[(size_t)c * ld + s];
      int b = ix[(size_t)c * ld + (s + 1) % ns];
      int p = fill[a]++;
      edge_cell[p] = c;
      edge_side[p] = s;
      edge_end[p] = b;
    }
  }
  for (size_t i = 0; i < (size_t)numel * nshared; ++i) nelcon[i] = -1;
  for (int c = 0; c < numel; ++c) {
    int ns = cell_sides(ix, ld, c, nshared);
    for (int s = 0; s < ns; ++s) {
      int a = ix[(size_t)c * ld + s];
      int b = ix[(size_t)c * ld + (s + 1) % ns];
      for (int p = off[b]; p < off[b + 1]; ++p) {
        if (edge_end[p] == a && edge_cell[p] != c) {
          nelcon[(size_t)c * nshared + s] = edge_cell[p] + 1;
          break;
        }
      }
    }
  }
  return FVC_OK;
}

int32_t fvc_mesh_rcm(const int32_t *nelcon, int32_t numel, int32_t nshared,
                     int32_t freord, int32_t *num) {
  if (!nelcon || !num || numel <= 0 || nshared <= 0) return FVC_ERR_ARG;
  if (!freord) {
    for (int i = 0; i < numel; ++i) num[i] = i + 1;
    return FVC_OK;
  }
  CellGraph g = graph_from_nelcon(nelcon, numel, nshared);
  Rcm rcm(g);
  std::vector<int> order = rcm.run();
  if ((int)order.size() != numel) return FVC_ERR_ARG;
  for (int k = 0; k < numel; ++k) num[order[k]] = k + 1;
  return FVC_OK;
}

int32_t fvc_mesh_numeq(const int32_t *num, const int32_t *nelcon,
                       int32_t numel, int32_t nshared, int32_t *id) {
  if (!num || !nelcon || !id || numel <= 0) return FVC_ERR_ARG;
  for (int c = 0; c < numel; ++c) {
    int n = num[c] - 1;
    if (n < 0 || n >= numel) return FVC_ERR_ARG;
    for (int j = 0; j < nshared; ++j) {
      int v = nelcon[(size_t)c * nshared + j];
      id[(size_t)n * nshared + j] = (v != -1) ? num[v - 1] : -1;
    }
  }
  return FVC_OK;
}

int32_t fvc_mesh_datastruc(const int32_t *id, int32_t neq, int32_t nshared,
                           int32_t matriz, int32_t unsym, int32_t *ia,
                           int32_t *ja, int32_t *nad, int64_t *ja_len) {
  if (!id || !ia || !nad || neq <= 0 || nshared <= 0) return FVC_ERR_ARG;
  if (matriz == 4) {
    int32_t count = 0;
    for (size_t q = 0; q < (size_t)neq * nshared; ++q)
      if (id[q] != -1) ++count;
    *nad = count;
    if (ja_len) *ja_len = (int64_t)neq * nshared;
    ia[0] = nshared;
    ia[1] = neq + 1;
    if (ja)
      for (size_t q = 0; q < (size_t)neq * nshared; ++q)
        ja[q] = (id[q] == -1) ? 1 : id[q];
    return FVC_OK;
  }
  bool lower, upper, diag;
  if (matriz == 1) {
    lower = true;
    upper = unsym != 0;
    diag = false;
  } else if (matriz == 2) {
    lower = upper = diag = true;
  } else if (matriz == 3) {
    lower = true;
    upper = false;
    diag = false;
  } else {
    return FVC_ERR_UNSUPPORTED;
  }
  auto keep = [&](int row, int v) {
    return v != -1 && ((lower && v < row) || (upper && v > row));
  };
  ia[0] = 1;
  for (int i = 0; i < neq; ++i) {
    int row = i + 1, c = diag ? 1 : 0;
    for (int j = 0; j < nshared; ++j)
      if (keep(row, id[(size_t)i * nshared + j])) ++c;
    ia[i + 1] = ia[i] + c;
  }
  *nad = ia[neq] - 1;
  if (ja_len) *ja_len = *nad;
  if (!ja) return FVC_OK;
  for (int i = 0; i < neq; ++i) {
    int row = i + 1;
    int p = ia[i] - 1;
    int start = p;
    if (diag) ja[p++] = row;
    for (int j = 0; j < nshared; ++j) {
      int v = id[(size_t)i * nshared + j];
      if (keep(row, v)) ja[p++] = v;
    }
    // CSR (matriz 2) keeps the diagonal first and faces in face order
    // (src/Datastruct.f:96-99); the other formats are sorted per row.
    if (matriz != 2) std::sort(ja + start, ja + p);
  }
  return FVC_OK;
}

}  // extern "C"
