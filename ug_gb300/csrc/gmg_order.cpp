// UG's ordering numprocs (np/procs/order.cc) on a flattened level.  UG runs
// them on its grid before the solve (the order of a level's VECTOR list is
// the order in which Gauss-Seidel and ILU visit the rows: l_setindex,
// ugiter.cc:169); here they run on the host over a gmg_level_desc before
// gmg_mg_create, and return the permutation that the caller applies to the
// level's rows (and to P's rows and the next finer P's columns).  Both are
// setup work of a few milliseconds, like UG's.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gmg_internal.h"

namespace {

int check_level_desc(const gmg_level_desc *L, int *perm) {
  GMG_CHECK(L && perm && L->n > 0 && L->rowptr && L->col, "order: an empty or incomplete level");
  const int n = L->n;
  GMG_CHECK(L->rowptr[0] == 0, "order: rowptr[0] != 0");
  for (int i = 0; i < n; ++i) {
    GMG_CHECK(L->rowptr[i + 1] >= L->rowptr[i], "order: rowptr decreases at row %d", i);
    for (int e = L->rowptr[i]; e < L->rowptr[i + 1]; ++e)
      GMG_CHECK(L->col[e] >= 0 && L->col[e] < n, "order: column %d of row %d out of range", L->col[e], i);
  }
  return 0;
}

}  // namespace

extern "C" {

// order.bw, OrderBW (order.cc:343-413): a breadth-first sweep from the first
// vector over the matrix graph (each row's entries in stored order, the
// diagonal skipped as MNEXT(VSTART(v)) skips it) finds the vector reached
// last; a second breadth-first sweep from that vector is the new order.  The
// bandwidth is max |i - j| over the entries in the new numbering.
int gmg_order_bw(const gmg_level_desc *L, int *perm, int *bandwidth) {
  if (check_level_desc(L, perm)) return 1;
  const int n = L->n;
  const int *rp = L->rowptr, *col = L->col;
  std::vector<char> used(n, 0);
  std::vector<int> fifo;
  fifo.reserve(n);
  fifo.push_back(0);
  used[0] = 1;
  int last = 0;
  for (size_t head = 0; head < fifo.size(); ++head) {
    last = fifo[head];
    for (int e = rp[last]; e < rp[last + 1]; ++e) {
      const int w = col[e];
      if (w != last && !used[w]) {
        used[w] = 1;
        fifo.push_back(w);
      }
    }
  }
  // the second sweep takes the vectors the first one marked and unmarks them
  fifo.clear();
  fifo.push_back(last);
  used[last] = 0;
  for (size_t head = 0; head < fifo.size(); ++head) {
    const int v = fifo[head];
    for (int e = rp[v]; e < rp[v + 1]; ++e) {
      const int w = col[e];
      if (w != v && used[w]) {
        used[w] = 0;
        fifo.push_back(w);
      }
    }
  }
  // UG asserts that every vector was reached (order.cc:394)
  GMG_CHECK((int)fifo.size() == n, "order bw: the matrix graph is not connected (%d of %d vectors reached)",
            (int)fifo.size(), n);
  std::vector<int> pos(n);
  for (int i = 0; i < n; ++i) {
    perm[i] = fifo[i];
    pos[fifo[i]] = i;
  }
  if (bandwidth) {
    int bw = 0;
    for (int v = 0; v < n; ++v)
      for (int e = rp[v]; e < rp[v + 1]; ++e) bw = std::max(bw, std::abs(pos[v] - pos[col[e]]));
    *bandwidth = bw;
  }
  return 0;
}

// order.lex, OrderLex (order.cc:287) -> LexOrderVectorsInGrid
// (gm/algebra.cc:4699-4790) with UG's settings (cartesian, every vector, no
// special place for skip vectors, matrices left in place).  config has one
// letter per dimension: r/l = x ascending/descending, u/d = y, f/b = z; the
// LAST letter is the most significant key.  Two positions compare by the
// differences scaled by inv_mesh_size (UG: 2^level * NN(level 0)^(1/dim) /
// the domain radius); a difference of at most 1e-3 in a key counts as equal
// and passes to the next key (LexCompare, algebra.cc:4533).
int gmg_order_lex(const gmg_level_desc *L, int dim, const double *xyz, int xyz_stride, const char *config,
                  double inv_mesh_size, int *perm) {
  GMG_CHECK(L && perm && L->n > 0 && xyz && config, "order lex: missing arguments");
  GMG_CHECK(dim == 2 || dim == 3, "order lex: dimension %d", dim);
  GMG_CHECK(xyz_stride >= dim, "order lex: coordinate stride %d below the dimension %d", xyz_stride, dim);
  GMG_CHECK(inv_mesh_size > 0.0 && std::isfinite(inv_mesh_size), "order lex: inv_mesh_size must be positive");
  GMG_CHECK((int)std::strlen(config) == dim, "order lex: config '%s' needs %d letters", config, dim);
  int ord[3], sign[3];
  for (int i = 0; i < dim; ++i) {  // OrderLexInit, order.cc:228-274
    switch (config[i]) {
      case 'r': ord[i] = 0; sign[i] = 1; break;
      case 'l': ord[i] = 0; sign[i] = -1; break;
      case 'u': ord[i] = 1; sign[i] = 1; break;
      case 'd': ord[i] = 1; sign[i] = -1; break;
      case 'f': GMG_CHECK(dim == 3, "order lex: 'f' needs 3 dimensions"); ord[i] = 2; sign[i] = 1; break;
      case 'b': GMG_CHECK(dim == 3, "order lex: 'b' needs 3 dimensions"); ord[i] = 2; sign[i] = -1; break;
      default: GMG_CHECK(false, "order lex: config letter '%c'", config[i]);
    }
  }
  const double res = 1e-3;  // ORDERRES, algebra.cc:114
  auto cmp = [&](int a, int b) {
    double diff[3];
    for (int d = 0; d < dim; ++d) diff[d] = (xyz[size_t(b) * xyz_stride + d] - xyz[size_t(a) * xyz_stride + d]) * inv_mesh_size;
    if (std::fabs(diff[ord[dim - 1]]) <= res) {
      if (dim == 3 && std::fabs(diff[ord[dim - 2]]) <= res) return diff[ord[0]] > 0.0 ? -sign[0] : sign[0];
      return diff[ord[dim - 2]] > 0.0 ? -sign[dim - 2] : sign[dim - 2];
    }
    return diff[ord[dim - 1]] > 0.0 ? -sign[dim - 1] : sign[dim - 1];
  };
  const int n = L->n;
  for (int i = 0; i < n; ++i) perm[i] = i;
  // LexCompare never reports equality; on distinct positions it is a strict
  // total order, so any correct sort gives UG's qsort result
  std::stable_sort(perm, perm + n, [&](int a, int b) { return cmp(a, b) < 0; });
  return 0;
}

}  // extern "C"
