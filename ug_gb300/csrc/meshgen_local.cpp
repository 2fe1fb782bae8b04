// Locally refined hierarchies: plane-strain P1 elasticity on the L-shaped
// domain (-1,1)^2 minus [0,1)x(-1,0], refined toward the re-entrant corner.
//
// The hierarchy is built the way UG's grid manager builds it (gm/refine.cc,
// gm/rm.cc, gm/ugm.cc, gm/algebra.cc), from the set of red-refined elements:
//   * coarse grid: the six triangles of the three unit squares, each split
//     by its diagonal through the corner (0, 0), corners counter-clockwise;
//   * a refinement step marks leaf elements; a mark goes to the element's
//     first RED_CLASS ancestor (ELEMENT_TO_MARK, rm.cc:2887);
//   * closure level by level (SetElementRules / Patterns2Rules, rm.cc:2674):
//     an edge of level l is refined if a red-refined element of level l has
//     it; a RED_CLASS element with pattern 7 turns red, patterns 1/2/4 take
//     T_BISECT_1_x, patterns 3/5/6 T_BISECT_2_T1_x (sons in the corner order
//     of UG's TriangleRules); a GREEN or YELLOW element with a refined edge
//     sends the red mark to its RED_CLASS ancestor, and the closure restarts
//     on that ancestor's level;
//   * copies (ComputeCopies, refine.cc:2865): next node class 3 on the
//     corners of refined elements, propagated twice over elements
//     (PropagateNextNodeClasses); an unrefined element with a corner of
//     next class >= 2 (MINVNCLASS) gets a yellow copy on the next level;
//   * node classes of a new level (refine.cc:6750-6782): 3 on the corners of
//     RED and GREEN elements, propagated twice over elements;
//   * vector classes (SetSurfaceClasses, algebra.cc:2838): VCLASS 3 on the
//     vectors of elements whose corners all have node class 3 (levels >= 1;
//     3 everywhere on level 0), VNCLASS 3 on those of elements whose corners
//     all have next node class 3 (0 on the top level), each propagated twice
//     over the matrix graph (3 -> 2 -> 1).
// Every level is assembled on all of its elements (red, green and yellow)
// with homogeneous Dirichlet rows on the boundary; the transfer weights are
// UG's standard ones (corner copy 1, edge midpoint 1/2-1/2).  Vectors are
// numbered in the order of first appearance in the level's element list,
// each row's matrix list is the diagonal then ascending columns.  The
// right-hand side lives on the surface rows (FINE_GRID_DOF below the top
// level, NEW_DEFECT on it): f * h_l^2 with f uniform[-1,1] keyed by the
// node's lattice position (fields.h) and h_l = 2^-l.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <memory>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/ug_gb300.h"
#include "fields.h"
#include "gmg_internal.h"

namespace {

enum { YELLOW = 1, GREEN = 2, RED = 3 };
enum { R_NONE = 0, R_COPY = 1, R_GREEN = 2, R_RED = 3 };

struct Tri {
  int v[3];        // position ids, UG corner order
  int cls;         // YELLOW / GREEN / RED
  int father;      // index in the level below (-1 on level 0)
};

struct Key3 {
  int a, b, c;
  bool operator==(const Key3 &o) const { return a == o.a && b == o.b && c == o.c; }
};
struct Key3Hash {
  size_t operator()(const Key3 &k) const {
    uint64_t h = ugfx::mix64((uint64_t(uint32_t(k.a)) << 32) ^ uint32_t(k.b));
    return size_t(ugfx::mix64(h ^ uint32_t(k.c)));
  }
};
static Key3 key_of(const Tri &t) {
  int s[3] = {t.v[0], t.v[1], t.v[2]};
  std::sort(s, s + 3);
  return {s[0], s[1], s[2]};
}
static uint64_t edge_key(int a, int b) {
  if (a > b) std::swap(a, b);
  return (uint64_t(uint32_t(a)) << 32) | uint32_t(b);
}

struct Mesh {
  int lmax;                                   // lattice scale 2^lmax
  std::vector<std::array<int64_t, 2>> pos;    // lattice coordinates of position ids
  std::unordered_map<uint64_t, int> pos_id;
  std::vector<std::vector<Tri>> lev;          // elements per level
  std::vector<std::vector<int>> rule;         // refinement of each element (R_*), pattern in rule >> 2
  std::vector<std::unordered_set<Key3, Key3Hash>> red;  // red-refined elements per level

  int position(int64_t x, int64_t y) {
    const int64_t off = int64_t(1) << lmax;
    const uint64_t k = (uint64_t(x + off) << 32) | uint64_t(y + off);
    auto it = pos_id.find(k);
    if (it != pos_id.end()) return it->second;
    const int id = int(pos.size());
    pos.push_back({x, y});
    pos_id.emplace(k, id);
    return id;
  }
  int midpoint(int a, int b) { return position((pos[a][0] + pos[b][0]) / 2, (pos[a][1] + pos[b][1]) / 2); }
  bool in_red(int l, const Tri &t) const { return l < int(red.size()) && red[l].count(key_of(t)); }
};

// UG's triangle edges: 0 = (0,1), 1 = (1,2), 2 = (0,2)
static const int EDGE[3][2] = {{0, 1}, {1, 2}, {0, 2}};

// sons of a refinement rule in UG's corner numbering (corners 0-2, edge
// midpoints 3 = e0, 4 = e1, 5 = e2), TriangleRules in gm/rm.cc
static int sons(int rule_pattern, int son[4][3]) {
  static const int red[4][3] = {{0, 3, 5}, {3, 1, 4}, {4, 2, 5}, {3, 4, 5}};
  static const int b10[2][3] = {{0, 3, 2}, {3, 1, 2}}, b11[2][3] = {{0, 1, 4}, {0, 4, 2}},
                   b12[2][3] = {{0, 1, 5}, {5, 1, 2}};
  static const int t12[3][3] = {{0, 3, 2}, {3, 1, 4}, {3, 4, 2}}, t11[3][3] = {{0, 3, 5}, {3, 1, 5}, {5, 1, 2}},
                   t10[3][3] = {{0, 1, 4}, {0, 4, 5}, {5, 4, 2}};
  const int(*tab)[3] = nullptr;
  int n = 0;
  switch (rule_pattern) {
    case 7: tab = red; n = 4; break;
    case 1: tab = b10; n = 2; break;
    case 2: tab = b11; n = 2; break;
    case 4: tab = b12; n = 2; break;
    case 3: tab = t12; n = 3; break;  // edges 0, 1: T_BISECT_2_T1_2
    case 5: tab = t11; n = 3; break;  // edges 0, 2: T_BISECT_2_T1_1
    case 6: tab = t10; n = 3; break;  // edges 1, 2: T_BISECT_2_T1_0
    default: return 0;
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) son[i][j] = tab[i][j];
  return n;
}

// the first RED_CLASS ancestor (ELEMENT_TO_MARK): (level, index)
static std::pair<int, int> red_ancestor(const Mesh &M, int l, int i) {
  while (M.lev[l][i].cls != RED) { i = M.lev[l][i].father; --l; }
  return {l, i};
}

// next node classes of level l's positions from the refinement rules
static void next_node_classes(const Mesh &M, int l, const std::vector<int> &rule, std::unordered_map<int, int> &nn) {
  nn.clear();
  const auto &E = M.lev[l];
  for (size_t e = 0; e < E.size(); ++e)
    if ((rule[e] & 3) == R_RED || (rule[e] & 3) == R_GREEN)
      for (int c = 0; c < 3; ++c) nn[E[e].v[c]] = 3;
  for (int cl = 3; cl >= 2; --cl) {  // PropagateNextNodeClass(3), then (2)
    std::vector<int> touched;
    for (const Tri &t : E) {
      int mx = 0;
      for (int c = 0; c < 3; ++c) { auto it = nn.find(t.v[c]); if (it != nn.end()) mx = std::max(mx, it->second); }
      if (mx != cl) continue;
      for (int c = 0; c < 3; ++c) {
        auto it = nn.find(t.v[c]);
        if (it == nn.end() || it->second < cl) touched.push_back(t.v[c]);
      }
    }
    for (int p : touched) { int &v = nn[p]; v = std::max(v, cl - 1); }
  }
}

// rebuilds the levels above the coarse grid from the red sets; returns the top level
static int build(Mesh &M) {
  M.lev.resize(1);
  M.rule.assign(1, {});
  int l = 0;
  for (;;) {
    const auto &E = M.lev[l];
    if (int(M.red.size()) <= l + 1) M.red.resize(l + 2);
    // closure on level l
    std::vector<int> rule(E.size(), R_NONE);
    int restart = -1;
    for (;;) {
      std::unordered_set<uint64_t> re;
      for (const Tri &t : E)
        if (t.cls == RED && M.in_red(l, t))
          for (auto &ed : EDGE) re.insert(edge_key(t.v[ed[0]], t.v[ed[1]]));
      bool changed = false;
      for (size_t e = 0; e < E.size() && restart < 0; ++e) {
        const Tri &t = E[e];
        int p = 0;
        for (int k = 0; k < 3; ++k)
          if (re.count(edge_key(t.v[EDGE[k][0]], t.v[EDGE[k][1]]))) p |= 1 << k;
        if (t.cls == RED) {
          if (M.in_red(l, t)) rule[e] = R_RED | (7 << 2);
          else if (p == 7) { M.red[l].insert(key_of(t)); changed = true; }
          else rule[e] = p ? (R_GREEN | (p << 2)) : R_NONE;
        } else if (p) {
          auto a = red_ancestor(M, l, int(e));
          if (!M.red[a.first].count(key_of(M.lev[a.first][a.second]))) {
            M.red[a.first].insert(key_of(M.lev[a.first][a.second]));
            restart = a.first;
          }
        }
      }
      if (restart >= 0 || !changed) break;
    }
    if (restart >= 0) {
      // the red set of a lower level grew: rebuild from there
      M.lev.resize(restart + 1);
      M.rule.resize(restart + 1);
      l = restart;
      continue;
    }
    // copies
    bool any = false;
    for (int r : rule) any |= (r & 3) != R_NONE;
    if (!any) { M.rule.resize(l + 1); M.rule[l] = rule; return l; }
    std::unordered_map<int, int> nn;
    next_node_classes(M, l, rule, nn);
    for (size_t e = 0; e < E.size(); ++e) {
      if ((rule[e] & 3) != R_NONE) continue;
      int mx = 0;
      for (int c = 0; c < 3; ++c) { auto it = nn.find(E[e].v[c]); if (it != nn.end()) mx = std::max(mx, it->second); }
      if (mx >= 2) rule[e] = R_COPY;
    }
    M.rule.resize(l + 1);
    M.rule[l] = rule;
    // level l + 1
    std::vector<Tri> F;
    for (size_t e = 0; e < E.size(); ++e) {
      const Tri &t = E[e];
      const int kind = rule[e] & 3;
      if (kind == R_NONE) continue;
      if (kind == R_COPY) { F.push_back({{t.v[0], t.v[1], t.v[2]}, YELLOW, int(e)}); continue; }
      const int pattern = rule[e] >> 2;
      int node[6] = {t.v[0], t.v[1], t.v[2], -1, -1, -1};
      for (int k = 0; k < 3; ++k)
        if (pattern & (1 << k)) node[3 + k] = M.midpoint(t.v[EDGE[k][0]], t.v[EDGE[k][1]]);
      int sn[4][3];
      const int ns = sons(pattern, sn);
      for (int i = 0; i < ns; ++i)
        F.push_back({{node[sn[i][0]], node[sn[i][1]], node[sn[i][2]]}, kind == R_RED ? RED : GREEN, int(e)});
    }
    M.lev.push_back(std::move(F));
    ++l;
  }
}

struct Level {
  int n = 0;
  std::vector<int> node;                  // level vector -> position id
  std::unordered_map<int, int> idx;       // position id -> level vector
  std::vector<std::vector<int>> adj;      // matrix graph (without the diagonal)
  std::vector<int> ncl, nncl, vclass, vnclass;
};

static void propagate_vectors(const Level &L, std::vector<int> &cls) {
  for (int c = 3; c >= 2; --c) {  // PropagateVectorClass(3), then (2)
    std::vector<int> set;
    for (int i = 0; i < L.n; ++i)
      if (cls[i] == c)
        for (int j : L.adj[i])
          if (cls[j] < c) set.push_back(j);
    for (int j : set) cls[j] = std::max(cls[j], c - 1);
  }
}

static void node_classes_of(const std::vector<Tri> &E, const Level &L, const std::vector<char> &seed,
                            std::vector<int> &cls) {
  cls.assign(L.n, 0);
  for (size_t e = 0; e < E.size(); ++e)
    if (seed[e])
      for (int c = 0; c < 3; ++c) cls[L.idx.at(E[e].v[c])] = 3;
  for (int cl = 3; cl >= 2; --cl) {
    std::vector<int> set;
    for (const Tri &t : E) {
      int mx = 0;
      for (int c = 0; c < 3; ++c) mx = std::max(mx, cls[L.idx.at(t.v[c])]);
      if (mx != cl) continue;
      for (int c = 0; c < 3; ++c) {
        int i = L.idx.at(t.v[c]);
        if (cls[i] < cl) set.push_back(i);
      }
    }
    for (int i : set) cls[i] = std::max(cls[i], cl - 1);
  }
}

static void elast_block(const double X[3][2], double K[3][3][4]) {
  const double nu = 0.3, E = 1.0;
  const double lam = E * nu / ((1 + nu) * (1 - 2 * nu)), mu = E / (2 * (1 + nu));
  double J00 = X[1][0] - X[0][0], J01 = X[2][0] - X[0][0], J10 = X[1][1] - X[0][1], J11 = X[2][1] - X[0][1];
  double det = J00 * J11 - J01 * J10;
  double i00 = J11 / det, i01 = -J01 / det, i10 = -J10 / det, i11 = J00 / det;
  double G[3][2] = {{-(i00 + i10), -(i01 + i11)}, {i00, i01}, {i10, i11}};
  double area = std::fabs(det) / 2.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double gg = G[i][0] * G[j][0] + G[i][1] * G[j][1];
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
          K[i][j][a * 2 + b] = area * (lam * G[i][a] * G[j][b] + mu * G[i][b] * G[j][a] + (a == b ? mu * gg : 0.0));
    }
}

}  // namespace

struct gmg_lgen {
  std::vector<std::vector<int>> rowptr, col, vclass, vnclass, skip, prow, pcol;
  std::vector<std::vector<double>> val, pw, xyz;
  std::vector<gmg_level_desc> desc;
  std::vector<double> rhs;  // every level, concatenated
  int frl = 0;
};

extern "C" {

int gmg_lgen_create(int nuni, int nloc, unsigned long long seed, gmg_lgen **out) {
  if (!out || nuni < 0 || nloc < 0 || nuni + nloc > 20) {
    gmg::set_error("gmg_lgen_create: bad arguments (nuni %d, nloc %d)", nuni, nloc);
    return 1;
  }
  *out = nullptr;
  Mesh M;
  M.lmax = nuni + nloc;
  const int64_t one = int64_t(1) << M.lmax;
  const int64_t C[8][2] = {{-1, -1}, {0, -1}, {0, 0}, {1, 0}, {1, 1}, {0, 1}, {-1, 1}, {-1, 0}};
  int cid[8];
  for (int i = 0; i < 8; ++i) cid[i] = M.position(C[i][0] * one, C[i][1] * one);
  const int T[6][3] = {{0, 1, 2}, {0, 2, 7}, {7, 2, 6}, {2, 5, 6}, {2, 3, 4}, {2, 4, 5}};
  M.lev.assign(1, {});
  for (auto &t : T) M.lev[0].push_back({{cid[t[0]], cid[t[1]], cid[t[2]]}, RED, -1});
  M.red.assign(1, {});
  int top = build(M);
  // uniform steps: every element of the top level; local steps: leaves near the corner
  for (int step = 0; step < nuni + nloc; ++step) {
    std::vector<std::pair<int, int>> marks;
    const bool local = step >= nuni;
    const double r = local ? std::ldexp(1.0, -(step - nuni + 1)) : 0.0;
    for (int l = 0; l <= top; ++l)
      for (size_t e = 0; e < M.lev[l].size(); ++e) {
        if (l < top && (M.rule[l][e] & 3) != R_NONE) continue;  // not a leaf
        if (!local && l != top) continue;
        bool near = !local;
        for (int c = 0; c < 3 && !near; ++c) {
          const double x = double(M.pos[M.lev[l][e].v[c]][0]) / double(one);
          const double y = double(M.pos[M.lev[l][e].v[c]][1]) / double(one);
          near = x * x + y * y <= r * r;
        }
        if (near) marks.push_back(red_ancestor(M, l, int(e)));
      }
    for (auto &m : marks) {
      if (int(M.red.size()) <= m.first) M.red.resize(m.first + 1);
      M.red[m.first].insert(key_of(M.lev[m.first][m.second]));
    }
    top = build(M);
  }
  const int nl = top + 1;
  // vectors, classes, matrices
  std::vector<Level> L(nl);
  for (int l = 0; l < nl; ++l) {
    Level &V = L[l];
    for (const Tri &t : M.lev[l])
      for (int c = 0; c < 3; ++c)
        if (V.idx.emplace(t.v[c], V.n).second) { V.node.push_back(t.v[c]); ++V.n; }
    std::vector<std::unordered_set<int>> adj(V.n);
    for (const Tri &t : M.lev[l])
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          if (a != b) adj[V.idx[t.v[a]]].insert(V.idx[t.v[b]]);
    V.adj.resize(V.n);
    for (int i = 0; i < V.n; ++i) {
      V.adj[i].assign(adj[i].begin(), adj[i].end());
      std::sort(V.adj[i].begin(), V.adj[i].end());
    }
    std::vector<char> seed_nc(M.lev[l].size()), seed_nn(M.lev[l].size());
    for (size_t e = 0; e < M.lev[l].size(); ++e) {
      seed_nc[e] = M.lev[l][e].cls >= GREEN;
      seed_nn[e] = l < top && ((M.rule[l][e] & 3) == R_RED || (M.rule[l][e] & 3) == R_GREEN);
    }
    node_classes_of(M.lev[l], V, seed_nc, V.ncl);
    node_classes_of(M.lev[l], V, seed_nn, V.nncl);
    // SetSurfaceClasses
    V.vclass.assign(V.n, l == 0 ? 3 : 0);
    V.vnclass.assign(V.n, 0);
    for (const Tri &t : M.lev[l]) {
      int mn = 3, mnn = 3;
      for (int c = 0; c < 3; ++c) {
        const int i = V.idx[t.v[c]];
        mn = std::min(mn, V.ncl[i]);
        mnn = std::min(mnn, V.nncl[i]);
      }
      if (l > 0 && mn == 3)
        for (int c = 0; c < 3; ++c) V.vclass[V.idx[t.v[c]]] = 3;
      if (l < top && mnn == 3)
        for (int c = 0; c < 3; ++c) V.vnclass[V.idx[t.v[c]]] = 3;
    }
    if (l > 0) propagate_vectors(V, V.vclass);
    if (l < top) propagate_vectors(V, V.vnclass);
  }
  auto G = std::make_unique<gmg_lgen>();
  G->rowptr.resize(nl); G->col.resize(nl); G->vclass.resize(nl); G->vnclass.resize(nl); G->skip.resize(nl);
  G->prow.resize(nl); G->pcol.resize(nl); G->val.resize(nl); G->pw.resize(nl); G->xyz.resize(nl);
  const int s = 2, ss = 4;
  for (int l = 0; l < nl; ++l) {
    Level &V = L[l];
    auto &rp = G->rowptr[l];
    auto &cl = G->col[l];
    rp.assign(V.n + 1, 0);
    for (int i = 0; i < V.n; ++i) rp[i + 1] = rp[i] + 1 + int(V.adj[i].size());
    cl.resize(rp[V.n]);
    for (int i = 0; i < V.n; ++i) {
      cl[rp[i]] = i;
      std::copy(V.adj[i].begin(), V.adj[i].end(), cl.begin() + rp[i] + 1);
    }
    auto &val = G->val[l];
    val.assign(size_t(rp[V.n]) * ss, 0.0);
    auto entry = [&](int i, int j) -> double * {
      if (i == j) return &val[size_t(rp[i]) * ss];
      const auto &a = V.adj[i];
      const int k = int(std::lower_bound(a.begin(), a.end(), j) - a.begin());
      return &val[size_t(rp[i] + 1 + k) * ss];
    };
    for (const Tri &t : M.lev[l]) {
      double X[3][2];
      for (int c = 0; c < 3; ++c) {
        X[c][0] = double(M.pos[t.v[c]][0]) / double(one);
        X[c][1] = double(M.pos[t.v[c]][1]) / double(one);
      }
      double K[3][3][4];
      elast_block(X, K);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          double *m = entry(V.idx[t.v[a]], V.idx[t.v[b]]);
          for (int q = 0; q < ss; ++q) m[q] += K[a][b][q];
        }
    }
    // Dirichlet: the whole boundary of the L
    auto &sk = G->skip[l];
    sk.assign(V.n, 0);
    auto &xyz = G->xyz[l];
    xyz.assign(size_t(V.n) * 3, 0.0);
    for (int i = 0; i < V.n; ++i) {
      const int64_t x = M.pos[V.node[i]][0], y = M.pos[V.node[i]][1];
      xyz[size_t(i) * 3] = double(x) / double(one);
      xyz[size_t(i) * 3 + 1] = double(y) / double(one);
      const bool bnd = x == -one || x == one || y == -one || y == one || (x == 0 && y <= 0) || (y == 0 && x >= 0);
      if (!bnd) continue;
      sk[i] = 3;
      for (int k = rp[i]; k < rp[i + 1]; ++k)
        for (int q = 0; q < ss; ++q) val[size_t(k) * ss + q] = (k == rp[i] && (q == 0 || q == 3)) ? 1.0 : 0.0;
    }
    G->vclass[l] = V.vclass;
    G->vnclass[l] = V.vnclass;
    if (l == 0) continue;
    // standard transfer: corner copy or edge midpoint
    const Level &Cs = L[l - 1];
    auto &pr = G->prow[l];
    auto &pc = G->pcol[l];
    auto &pw = G->pw[l];
    pr.assign(1, 0);
    std::unordered_map<int, std::pair<int, int>> mid;  // midpoint position -> father edge
    for (size_t e = 0; e < M.lev[l - 1].size(); ++e) {
      const int pattern = M.rule[l - 1][e] >> 2;
      const Tri &t = M.lev[l - 1][e];
      for (int k = 0; k < 3; ++k)
        if (pattern & (1 << k)) {
          const int a = t.v[EDGE[k][0]], b = t.v[EDGE[k][1]];
          mid.emplace(M.midpoint(a, b), std::make_pair(a, b));
        }
    }
    for (int i = 0; i < V.n; ++i) {
      auto c = Cs.idx.find(V.node[i]);
      if (c != Cs.idx.end()) {
        pc.push_back(c->second); pw.push_back(1.0);
      } else {
        const auto &ab = mid.at(V.node[i]);
        pc.push_back(Cs.idx.at(ab.first)); pw.push_back(0.5);
        pc.push_back(Cs.idx.at(ab.second)); pw.push_back(0.5);
      }
      pr.push_back(int(pc.size()));
    }
  }
  // FULLREFINELEVEL and the right-hand side on the surface
  G->frl = top;
  for (int l = top; l >= 0; --l)
    for (int i = 0; i < L[l].n; ++i)
      if (L[l].vclass[i] >= 2 && L[l].vnclass[i] <= 1) { G->frl = l; break; }
  for (int l = 0; l < nl; ++l) {
    const double hd = std::ldexp(1.0, -2 * l);
    for (int i = 0; i < L[l].n; ++i) {
      const bool surf = l == top ? L[l].vclass[i] >= 2
                                 : (l >= G->frl && L[l].vclass[i] >= 2 && L[l].vnclass[i] <= 1);
      // lattice position on the top level's grid (spacing 2^-top)
      const int64_t x = M.pos[L[l].node[i]][0], y = M.pos[L[l].node[i]][1];
      const uint64_t key = ugfx::lattice_key((x + one) >> (M.lmax - top), (y + one) >> (M.lmax - top), 0);
      for (int c = 0; c < s; ++c)
        G->rhs.push_back(surf && !(G->skip[l][i] & (1 << c)) ? ugfx::rhs_uniform(seed + 0x9E37ull * c, key) * hd
                                                             : 0.0);
    }
  }
  G->desc.resize(nl);
  for (int l = 0; l < nl; ++l) {
    gmg_level_desc &d = G->desc[l];
    d.n = L[l].n; d.s = s;
    d.rowptr = G->rowptr[l].data(); d.col = G->col[l].data(); d.val = G->val[l].data();
    d.vclass = G->vclass[l].data(); d.vnclass = G->vnclass[l].data(); d.skip = G->skip[l].data();
    d.prowptr = l ? G->prow[l].data() : nullptr;
    d.pcol = l ? G->pcol[l].data() : nullptr;
    d.pw = l ? G->pw[l].data() : nullptr;
  }
  *out = G.release();
  return 0;
}

int gmg_lgen_levels(gmg_lgen *g, const gmg_level_desc **levels, int *nlevels) {
  if (!g || !levels || !nlevels) return 1;
  *levels = g->desc.data();
  *nlevels = int(g->desc.size());
  return 0;
}

int gmg_lgen_rhs(gmg_lgen *g, const double **rhs, long long *len) {
  if (!g || !rhs || !len) return 1;
  *rhs = g->rhs.data();
  *len = (long long)g->rhs.size();
  return 0;
}

int gmg_lgen_coords(gmg_lgen *g, int level, const double **xyz) {
  if (!g || !xyz || level < 0 || level >= int(g->xyz.size())) return 1;
  *xyz = g->xyz[level].data();
  return 0;
}

int gmg_lgen_destroy(gmg_lgen *g) {
  delete g;
  return 0;
}

}  // extern "C"
