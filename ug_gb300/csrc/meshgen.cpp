// Structured multigrid hierarchies for the benchmark and test workloads.
//
// UG's uniform red refinement of the workloads' coarse grids yields
// structured meshes, so they can be generated directly instead of through
// the grid manager (which needs minutes and gigabytes at 3D level 6-7):
//   kind 0: unit square, one Q1 quadrilateral, refined nref times
//           (every cell a Q1 element);
//   kind 1: unit cube, six Kuhn tetrahedra around the main diagonal, refined
//           nref times: the Freudenthal triangulation of the cube grid (every
//           cell split into the six tetrahedra x_s1 >= x_s2 >= x_s3 of its
//           local coordinates), whose edges are the segments [x, x + e_S]
//           for nonempty coordinate subsets S;
//   kind 2: unit square, two triangles split along the (1,1) diagonal,
//           refined nref times: every cell split along its (1,1) diagonal.
// Each level is assembled on its own elements (as the exporter driving UG
// does), with homogeneous Dirichlet rows (unit diagonal block, zero
// off-diagonal blocks, VECSKIP on every component) on the boundary, and the
// standard transfer weights of the refinement (corner copy, edge midpoint
// 1/2-1/2, Q1 cell centre 1/4 each).  Vectors are numbered lexicographically
// (x fastest).  The right-hand side is attached to lattice positions
// (fields.h), so it matches the UG-built problem node by node.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "../../include/ug_gb300.h"
#include "fields.h"
#include "gmg_internal.h"

namespace {

struct GenLevel {
  int n = 0, s = 1, N = 0;  // N = points per axis
  std::vector<int> rowptr, col, vclass, vnclass, skip, prow, pcol;
  std::vector<double> val, pw, xyz;
  // kind 3: the six tetrahedra of every lattice cell ((z Nc + y) Nc + x) as
  // masks of the cell's corners (bit dx | dy << 1 | dz << 2), ascending
  std::vector<uint8_t> cell_masks;
};

struct Offs {
  int dim;
  std::vector<std::array<int, 3>> d;  // neighbour offsets (diagonal not included)
};

static Offs offsets(int kind) {
  Offs o;
  if (kind == 0) {
    o.dim = 2;
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx)
        if (dx || dy) o.d.push_back({dx, dy, 0});
  } else if (kind == 1) {
    o.dim = 3;
    for (int m = 1; m < 8; ++m) {
      int a = m & 1, b = (m >> 1) & 1, c = (m >> 2) & 1;
      o.d.push_back({a, b, c});
      o.d.push_back({-a, -b, -c});
    }
  } else {
    o.dim = 2;
    const int t[6][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}, {1, 1}, {-1, -1}};
    for (auto &v : t) o.d.push_back({v[0], v[1], 0});
  }
  return o;
}

struct Grid {
  int dim, N;
  int idx(int i, int j, int k) const { return dim == 2 ? j * N + i : (k * N + j) * N + i; }
  int count() const { return dim == 2 ? N * N : N * N * N; }
  bool inside(int i, int j, int k) const {
    return i >= 0 && j >= 0 && k >= 0 && i < N && j < N && (dim == 2 ? k == 0 : k < N);
  }
  bool boundary(int i, int j, int k) const {
    return i == 0 || j == 0 || i == N - 1 || j == N - 1 || (dim == 3 && (k == 0 || k == N - 1));
  }
};

// stiffness of one P1 simplex (dim+1 corners) scaled by kk, into K (row-major (dim+1)^2)
static void p1_stiffness(int dim, const double X[4][3], double kk, double *K) {
  double G[4][3] = {{0}};
  double det;
  if (dim == 2) {
    double J00 = X[1][0] - X[0][0], J01 = X[2][0] - X[0][0], J10 = X[1][1] - X[0][1], J11 = X[2][1] - X[0][1];
    det = J00 * J11 - J01 * J10;
    double i00 = J11 / det, i01 = -J01 / det, i10 = -J10 / det, i11 = J00 / det;
    G[1][0] = i00; G[1][1] = i01; G[2][0] = i10; G[2][1] = i11;
    G[0][0] = -(i00 + i10); G[0][1] = -(i01 + i11);
  } else {
    double J[3][3];
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) J[r][c] = X[c + 1][r] - X[0][r];
    det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    double Ji[3][3];
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det; Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det; Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det; Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det; Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    for (int d = 0; d < 3; ++d) {
      G[1][d] = Ji[0][d]; G[2][d] = Ji[1][d]; G[3][d] = Ji[2][d];
      G[0][d] = -(Ji[0][d] + Ji[1][d] + Ji[2][d]);
    }
  }
  const int nc = dim + 1;
  const double vol = std::fabs(det) / (dim == 2 ? 2.0 : 6.0);
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j < nc; ++j) {
      double a = 0;
      for (int d = 0; d < dim; ++d) a += G[i][d] * G[j][d];
      K[i * nc + j] = kk * vol * a;
    }
}

// plane-strain P1 elasticity block stiffness (E=1, nu=0.3), K[(i*3+j)*4 + a*2+b]
static void elast_stiffness(const double X[4][3], double *K) {
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
          K[(i * 3 + j) * 4 + a * 2 + b] = area * (lam * G[i][a] * G[j][b] + mu * G[i][b] * G[j][a] + (a == b ? mu * gg : 0.0));
    }
}

static int nthreads() {
  unsigned h = std::thread::hardware_concurrency();
  return h ? int(std::min(h, 64u)) : 4;
}

}  // namespace

struct gmg_gen {
  int kind = 0, nref = 0;
  std::vector<GenLevel> lev;
  std::vector<gmg_level_desc> desc;
  std::vector<double> rhs;
};

static int build_level(gmg_gen *G, int l, const ugfx::LogNormalField &field) {
  const int kind = G->kind;
  const Offs O = offsets(kind);
  const int dim = O.dim, s = kind == 2 ? 2 : 1, ss = s * s;
  Grid g{dim, (1 << l) + 1};
  GenLevel &L = G->lev[l];
  L.N = g.N;
  L.s = s;
  L.n = g.count();
  const int n = L.n, noff = int(O.d.size());
  const double h = 1.0 / (g.N - 1);
  // pattern: diagonal first, then the neighbour offsets present in the grid
  std::vector<int> slot(size_t(n) * noff, -1);
  L.rowptr.assign(n + 1, 0);
  L.col.clear();
  L.col.reserve(size_t(n) * (noff + 1));
  L.xyz.assign(size_t(n) * 3, 0.0);
  for (int k = 0; k < (dim == 3 ? g.N : 1); ++k)
    for (int j = 0; j < g.N; ++j)
      for (int i = 0; i < g.N; ++i) {
        int r = g.idx(i, j, k);
        L.xyz[size_t(r) * 3] = i * h; L.xyz[size_t(r) * 3 + 1] = j * h; L.xyz[size_t(r) * 3 + 2] = dim == 3 ? k * h : 0.0;
        L.col.push_back(r);
        for (int o = 0; o < noff; ++o) {
          int a = i + O.d[o][0], b = j + O.d[o][1], c = k + O.d[o][2];
          if (!g.inside(a, b, c)) continue;
          slot[size_t(r) * noff + o] = int(L.col.size());
          L.col.push_back(g.idx(a, b, c));
        }
        L.rowptr[r + 1] = int(L.col.size());
      }
  L.val.assign(L.col.size() * ss, 0.0);
  // entry position of (row at p, column at q) from the lattice offset q - p
  auto pos = [&](const int p[3], const int q[3]) -> size_t {
    int r = g.idx(p[0], p[1], p[2]);
    if (p[0] == q[0] && p[1] == q[1] && p[2] == q[2]) return size_t(L.rowptr[r]);
    for (int o = 0; o < noff; ++o)
      if (O.d[o][0] == q[0] - p[0] && O.d[o][1] == q[1] - p[1] && O.d[o][2] == q[2] - p[2])
        return size_t(slot[size_t(r) * noff + o]);
    return size_t(-1);
  };
  // assembly over cells, one slab of cells (a row in 2D, a z-layer in 3D) per task
  const int nc = g.N - 1;
  static const double KQ1[4][4] = {{4, -1, -2, -1}, {-1, 4, -1, -2}, {-2, -1, 4, -1}, {-1, -2, -1, 4}};
  // work split along the slowest axis; each worker owns whole rows of cells, so
  // concurrent additions into one matrix row only happen across the split lines:
  // workers process even slabs, then odd slabs (no two concurrent slabs touch)
  auto do_slab = [&](int t) {
    std::vector<double> K(64);
    if (kind == 0) {
      for (int i = 0; i < nc; ++i) {
        int P[4][3] = {{i, t, 0}, {i + 1, t, 0}, {i + 1, t + 1, 0}, {i, t + 1, 0}};
        double kf = 1.0;
        if (field.M) { double xc[3] = {(i + 0.5) * h, (t + 0.5) * h, 0}; kf = field.k(xc); }
        for (int a = 0; a < 4; ++a)
          for (int b = 0; b < 4; ++b) L.val[pos(P[a], P[b])] += kf * KQ1[a][b] / 6.0;
      }
    } else if (kind == 2) {
      for (int i = 0; i < nc; ++i) {
        int T[2][3][3] = {{{i, t, 0}, {i + 1, t, 0}, {i + 1, t + 1, 0}}, {{i, t, 0}, {i + 1, t + 1, 0}, {i, t + 1, 0}}};
        for (int e = 0; e < 2; ++e) {
          double X[4][3] = {{0}};
          for (int a = 0; a < 3; ++a) for (int d = 0; d < 2; ++d) X[a][d] = T[e][a][d] * h;
          elast_stiffness(X, K.data());
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
              size_t q = pos(T[e][a], T[e][b]) * 4;
              for (int m = 0; m < 4; ++m) L.val[q + m] += K[(a * 3 + b) * 4 + m];
            }
        }
      }
    } else {
      static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
      for (int j = 0; j < nc; ++j)
        for (int i = 0; i < nc; ++i)
          for (int p = 0; p < 6; ++p) {
            int V[4][3];
            V[0][0] = i; V[0][1] = j; V[0][2] = t;
            for (int a = 1; a < 4; ++a) {
              for (int d = 0; d < 3; ++d) V[a][d] = V[a - 1][d];
              V[a][perms[p][a - 1]] += 1;
            }
            double X[4][3], xc[3] = {0, 0, 0};
            for (int a = 0; a < 4; ++a)
              for (int d = 0; d < 3; ++d) { X[a][d] = V[a][d] * h; xc[d] += X[a][d] / 4; }
            p1_stiffness(3, X, field.k(xc), K.data());
            for (int a = 0; a < 4; ++a)
              for (int b = 0; b < 4; ++b) L.val[pos(V[a], V[b])] += K[a * 4 + b];
          }
    }
  };
  const int nslab = nc;  // slab index = y (2D) or z (3D)
  const int nt = std::max(1, std::min(nthreads(), nslab));
  for (int parity = 0; parity < 2; ++parity) {
    std::vector<std::thread> th;
    for (int w = 0; w < nt; ++w)
      th.emplace_back([&, w]() {
        for (int t = parity + 2 * w; t < nslab; t += 2 * nt) do_slab(t);
      });
    for (auto &x : th) x.join();
  }
  // Dirichlet rows, classes
  L.vclass.assign(n, 3);
  // VNCLASS: 3 under a refined level, 0 on the finest level (no sons), as UG sets it
  L.vnclass.assign(n, l < G->nref ? 3 : 0);
  L.skip.assign(n, 0);
  for (int k = 0; k < (dim == 3 ? g.N : 1); ++k)
    for (int j = 0; j < g.N; ++j)
      for (int i = 0; i < g.N; ++i) {
        if (!g.boundary(i, j, k)) continue;
        int r = g.idx(i, j, k);
        L.skip[r] = (1 << s) - 1;
        for (int q = L.rowptr[r]; q < L.rowptr[r + 1]; ++q)
          for (int m = 0; m < ss; ++m) L.val[size_t(q) * ss + m] = (q == L.rowptr[r] && m % (s + 1) == 0) ? 1.0 : 0.0;
      }
  // standard transfer from level l-1
  if (l > 0) {
    Grid gc{dim, (1 << (l - 1)) + 1};
    L.prow.assign(n + 1, 0);
    L.pcol.clear();
    L.pw.clear();
    for (int k = 0; k < (dim == 3 ? g.N : 1); ++k)
      for (int j = 0; j < g.N; ++j)
        for (int i = 0; i < g.N; ++i) {
          int r = g.idx(i, j, k);
          int odd[3] = {i & 1, j & 1, k & 1};
          if (kind == 0 && odd[0] && odd[1]) {  // Q1 cell centre
            for (int b = 0; b < 2; ++b)
              for (int a = 0; a < 2; ++a) {
                L.pcol.push_back(gc.idx((i - 1) / 2 + a, (j - 1) / 2 + b, 0));
                L.pw.push_back(0.25);
              }
          } else if (!odd[0] && !odd[1] && !odd[2]) {  // corner: father copy
            L.pcol.push_back(gc.idx(i / 2, j / 2, k / 2));
            L.pw.push_back(1.0);
          } else {  // midpoint of the coarse edge [p - e_S, p + e_S]
            L.pcol.push_back(gc.idx((i - odd[0]) / 2, (j - odd[1]) / 2, (k - odd[2]) / 2));
            L.pw.push_back(0.5);
            L.pcol.push_back(gc.idx((i + odd[0]) / 2, (j + odd[1]) / 2, (k + odd[2]) / 2));
            L.pw.push_back(0.5);
          }
          L.prow[r + 1] = int(L.pcol.size());
        }
  }
  return 0;
}

// ------------------------------------------------------------ kind 3: UG's red refinement
// The six Kuhn tetrahedra of the unit cube, in the corner order the workload
// inserts them (corner ids of the cube 0..7 as the Hexahedron domain numbers
// them; every one positively oriented, so UG keeps the order), refined by
// UG's red rules: each tetrahedron splits into its four corner tetrahedra and
// the four of its octahedron cut along the shortest interior diagonal,
// ties broken as UG breaks them; sons carry their corners in the order of
// UG's rule table, which fixes the next refinement's edge numbering.
namespace {

// edges of a tetrahedron and the sons of the red rules that cut the
// octahedron along the diagonal between the midpoints of edges (2, 4),
// (0, 5) and (1, 3); son corners 0..3 = the father's corners, 4 + e = the
// midpoint of edge e
const int kTetEdge[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
const int kRedSons[3][8][4] = {
    {{0, 4, 6, 7}, {4, 5, 8, 1}, {5, 6, 9, 2}, {7, 8, 9, 3}, {4, 6, 7, 8}, {4, 5, 6, 8}, {5, 6, 8, 9}, {6, 7, 8, 9}},
    {{5, 6, 9, 2}, {4, 5, 8, 1}, {7, 8, 9, 3}, {0, 4, 6, 7}, {4, 5, 6, 9}, {5, 8, 9, 4}, {4, 7, 8, 9}, {4, 6, 7, 9}},
    {{7, 8, 9, 3}, {4, 5, 8, 1}, {0, 4, 6, 7}, {5, 6, 9, 2}, {5, 7, 8, 9}, {4, 5, 7, 8}, {4, 5, 6, 7}, {5, 6, 7, 9}}};
const int kCube[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
const int kCoarse[6][4] = {{0, 1, 2, 6}, {0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 4, 5, 6}, {0, 5, 1, 6}};

struct Tet {
  int v[4][3];  // lattice coordinates of the corners, UG's corner order
};

// the rule of the shortest interior diagonal (gm/rm.cc:1567): index into
// kRedSons; lengths compared exactly on the lattice
int red_rule(const int P[10][3]) {
  auto d2 = [&](int a, int b) {
    long long t = 0;
    for (int d = 0; d < 3; ++d) t += (long long)(P[a][d] - P[b][d]) * (P[a][d] - P[b][d]);
    return t;
  };
  const long long d05 = d2(4, 9), d13 = d2(5, 7), d24 = d2(6, 8);
  const int flags = int(d05 < d13) | (int(d13 < d24) << 1) | (int(d24 < d05) << 2);
  switch (flags) {
    case 2: case 6: return 2;  // 1_3
    case 4: case 5: return 0;  // 2_4
    default: return 1;         // 0_5 (flags 0, 1, 3)
  }
}

std::vector<Tet> refine_red(const std::vector<Tet> &in) {
  std::vector<Tet> out(in.size() * 8);
  for (size_t t = 0; t < in.size(); ++t) {
    int P[10][3];
    for (int c = 0; c < 4; ++c)
      for (int d = 0; d < 3; ++d) P[c][d] = 2 * in[t].v[c][d];
    for (int e = 0; e < 6; ++e)
      for (int d = 0; d < 3; ++d) P[4 + e][d] = in[t].v[kTetEdge[e][0]][d] + in[t].v[kTetEdge[e][1]][d];
    const int r = red_rule(P);
    for (int q = 0; q < 8; ++q)
      for (int c = 0; c < 4; ++c)
        for (int d = 0; d < 3; ++d) out[t * 8 + q].v[c][d] = P[kRedSons[r][q][c]][d];
  }
  return out;
}

// the 26 lattice directions: the 14 of the Freudenthal stencil first (for
// m = 1..7 with bits x, y, z: +m, -m), then the other 12
std::vector<std::array<int, 3>> offsets26() {
  std::vector<std::array<int, 3>> o;
  for (int m = 1; m < 8; ++m) {
    const int a = m & 1, b = (m >> 1) & 1, c = (m >> 2) & 1;
    o.push_back({a, b, c});
    o.push_back({-a, -b, -c});
  }
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        if (!dx && !dy && !dz) continue;
        const bool same = (dx >= 0 && dy >= 0 && dz >= 0) || (dx <= 0 && dy <= 0 && dz <= 0);
        if (!same) o.push_back({dx, dy, dz});
      }
  return o;
}
int off_index(const std::vector<std::array<int, 3>> &o, int dx, int dy, int dz) {
  for (int q = 0; q < int(o.size()); ++q)
    if (o[q][0] == dx && o[q][1] == dy && o[q][2] == dz) return q;
  return -1;
}

// one level of the UG-refined cube from its tetrahedra; `coarse_mask` (the
// level below's neighbour masks, null on level 0) gives the transfer
int build_ug_level(gmg_gen *G, int l, std::vector<Tet> &tets, const std::vector<uint32_t> *coarse_mask,
                   std::vector<uint32_t> &mask, const ugfx::LogNormalField &field) {
  static const std::vector<std::array<int, 3>> O = offsets26();
  GenLevel &L = G->lev[l];
  const int N = (1 << l) + 1, n = N * N * N, nc = N - 1;
  L.N = N; L.s = 1; L.n = n;
  const double h = 1.0 / nc;
  auto id = [&](const int *v) { return (v[2] * N + v[1]) * N + v[0]; };
  // the neighbours of every node: the edges of the tetrahedra
  mask.assign(n, 0u);
  for (const Tet &t : tets)
    for (auto &e : kTetEdge) {
      const int *a = t.v[e[0]], *b = t.v[e[1]];
      mask[id(a)] |= 1u << off_index(O, b[0] - a[0], b[1] - a[1], b[2] - a[2]);
      mask[id(b)] |= 1u << off_index(O, a[0] - b[0], a[1] - b[1], a[2] - b[2]);
    }
  // rows: the diagonal, then the neighbours in the order of O
  std::vector<int> slot(size_t(n) * 26, -1);
  L.rowptr.assign(n + 1, 0);
  L.col.clear();
  L.xyz.assign(size_t(n) * 3, 0.0);
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        const int r = (k * N + j) * N + i;
        L.xyz[size_t(r) * 3] = i * h; L.xyz[size_t(r) * 3 + 1] = j * h; L.xyz[size_t(r) * 3 + 2] = k * h;
        L.col.push_back(r);
        for (int o = 0; o < 26; ++o) {
          if (!(mask[r] & (1u << o))) continue;
          slot[size_t(r) * 26 + o] = int(L.col.size());
          L.col.push_back(((k + O[o][2]) * N + (j + O[o][1])) * N + (i + O[o][0]));
        }
        L.rowptr[r + 1] = int(L.col.size());
      }
  L.val.assign(L.col.size(), 0.0);
  // every tetrahedron lies in one lattice cell (its corners differ by at most
  // one step): sorted by cell (z, y, x), then by its sorted corner ids, the
  // contributions to every entry are summed in one fixed order -- z layers of
  // cells with even index first, then odd ones (no two layers of one parity
  // share a node, so they are assembled in parallel)
  struct Key { int z, y, x; std::array<int, 4> ids; size_t t; };
  std::vector<Key> keys(tets.size());
  for (size_t t = 0; t < tets.size(); ++t) {
    Key &kk = keys[t];
    kk.x = std::min({tets[t].v[0][0], tets[t].v[1][0], tets[t].v[2][0], tets[t].v[3][0]});
    kk.y = std::min({tets[t].v[0][1], tets[t].v[1][1], tets[t].v[2][1], tets[t].v[3][1]});
    kk.z = std::min({tets[t].v[0][2], tets[t].v[1][2], tets[t].v[2][2], tets[t].v[3][2]});
    for (int c = 0; c < 4; ++c) kk.ids[c] = id(tets[t].v[c]);
    std::sort(kk.ids.begin(), kk.ids.end());
    kk.t = t;
  }
  std::sort(keys.begin(), keys.end(), [](const Key &a, const Key &b) {
    if (a.z != b.z) return a.z < b.z;
    if (a.y != b.y) return a.y < b.y;
    if (a.x != b.x) return a.x < b.x;
    return a.ids < b.ids;
  });
  // every cell holds six tetrahedra of volume h^3 / 6 (6 8^l of them fill the
  // 8^l cells, and a tetrahedron on cube corners has volume 1/6 or 1/3 of it):
  // their corner masks, the device assembly's description of the mesh
  L.cell_masks.assign(size_t(nc) * nc * nc * 6, 0);
  {
    std::vector<uint8_t> fill(size_t(nc) * nc * nc, 0);
    for (const Key &kk : keys) {
      const Tet &T = tets[kk.t];
      int mask = 0;
      for (int a = 0; a < 4; ++a)
        mask |= 1 << ((T.v[a][0] - kk.x) | ((T.v[a][1] - kk.y) << 1) | ((T.v[a][2] - kk.z) << 2));
      const size_t cell = (size_t(kk.z) * nc + kk.y) * nc + kk.x;
      if (fill[cell] >= 6) {
        gmg::set_error("UG cube level %d: more than six tetrahedra in cell (%d,%d,%d)", l, kk.x, kk.y, kk.z);
        return 1;
      }
      L.cell_masks[cell * 6 + fill[cell]++] = uint8_t(mask);
    }
    for (size_t c = 0; c < fill.size(); ++c) {
      if (fill[c] != 6) {
        gmg::set_error("UG cube level %d: cell %zu holds %d tetrahedra", l, c, int(fill[c]));
        return 1;
      }
      std::sort(L.cell_masks.begin() + c * 6, L.cell_masks.begin() + c * 6 + 6);
    }
  }
  std::vector<size_t> zbeg(nc + 1, 0);
  for (const Key &kk : keys) zbeg[kk.z + 1]++;
  for (int z = 0; z < nc; ++z) zbeg[z + 1] += zbeg[z];
  auto do_slab = [&](int z) {
    double K[16];
    for (size_t q = zbeg[z]; q < zbeg[z + 1]; ++q) {
      const Tet &T = tets[keys[q].t];
      double X[4][3], xc[3] = {0, 0, 0};
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) { X[a][d] = T.v[a][d] * h; xc[d] += X[a][d] / 4; }
      p1_stiffness(3, X, field.k(xc), K);
      for (int a = 0; a < 4; ++a) {
        const int r = id(T.v[a]);
        for (int b = 0; b < 4; ++b) {
          const int e = a == b ? L.rowptr[r]
                               : slot[size_t(r) * 26 + off_index(O, T.v[b][0] - T.v[a][0], T.v[b][1] - T.v[a][1],
                                                                  T.v[b][2] - T.v[a][2])];
          L.val[e] += K[a * 4 + b];
        }
      }
    }
  };
  const int nt = std::max(1, std::min(nthreads(), nc));
  for (int parity = 0; parity < 2; ++parity) {
    std::vector<std::thread> th;
    for (int w = 0; w < nt; ++w)
      th.emplace_back([&, w]() {
        for (int z = parity + 2 * w; z < nc; z += 2 * nt) do_slab(z);
      });
    for (auto &x : th) x.join();
  }
  // classes, Dirichlet rows
  L.vclass.assign(n, 3);
  L.vnclass.assign(n, l < G->nref ? 3 : 0);
  L.skip.assign(n, 0);
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        if (!(i == 0 || j == 0 || k == 0 || i == N - 1 || j == N - 1 || k == N - 1)) continue;
        const int r = (k * N + j) * N + i;
        L.skip[r] = 1;
        for (int q = L.rowptr[r]; q < L.rowptr[r + 1]; ++q) L.val[q] = q == L.rowptr[r] ? 1.0 : 0.0;
      }
  // standard transfer: a corner copies its father; any other node is the
  // midpoint of the one coarse edge among the segments through it
  if (coarse_mask) {
    const int Nc = (1 << (l - 1)) + 1;
    L.prow.assign(n + 1, 0);
    L.pcol.clear();
    L.pw.clear();
    for (int k = 0; k < N; ++k)
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          const int r = (k * N + j) * N + i, odd[3] = {i & 1, j & 1, k & 1}, c[3] = {i / 2, j / 2, k / 2};
          if (!odd[0] && !odd[1] && !odd[2]) {
            L.pcol.push_back((c[2] * Nc + c[1]) * Nc + c[0]);
            L.pw.push_back(1.0);
          } else {
            int found = 0;
            for (int sg = 0; sg < 8 && !found; ++sg) {  // the low end of the segment: (p - e) / 2 per odd axis
              int lo[3], hi[3];
              bool ok = true;
              for (int d = 0; d < 3; ++d) {
                const int pd = d == 0 ? i : d == 1 ? j : k;
                if (!odd[d]) { lo[d] = hi[d] = pd / 2; if ((sg >> d) & 1) ok = false; continue; }
                const int sgn = ((sg >> d) & 1) ? -1 : 1;
                lo[d] = (pd - sgn) / 2;
                hi[d] = (pd + sgn) / 2;
              }
              if (!ok) continue;
              const int a = (lo[2] * Nc + lo[1]) * Nc + lo[0];
              const int q = off_index(O, hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]);
              if (q >= 0 && ((*coarse_mask)[a] & (1u << q))) {
                L.pcol.push_back(a); L.pw.push_back(0.5);
                L.pcol.push_back((hi[2] * Nc + hi[1]) * Nc + hi[0]); L.pw.push_back(0.5);
                found = 1;
              }
            }
            if (!found) {
              gmg::set_error("UG cube level %d: node (%d,%d,%d) is on no coarse edge", l, i, j, k);
              return 1;
            }
          }
          L.prow[r + 1] = int(L.pcol.size());
        }
  }
  return 0;
}

int build_ug_cube(gmg_gen *G, const ugfx::LogNormalField &field) {
  std::vector<Tet> tets(6);
  for (int t = 0; t < 6; ++t)
    for (int c = 0; c < 4; ++c)
      for (int d = 0; d < 3; ++d) tets[t].v[c][d] = kCube[kCoarse[t][c]][d];
  std::vector<uint32_t> mask, prev;
  for (int l = 0; l <= G->nref; ++l) {
    if (l > 0) tets = refine_red(tets);
    if (build_ug_level(G, l, tets, l > 0 ? &prev : nullptr, mask, field)) return 1;
    prev.swap(mask);
  }
  return 0;
}

}  // namespace

namespace gmg {
const uint8_t *gen_cell_masks(const gmg_gen *g, int level) {
  if (!g || level < 0 || level > g->nref || g->lev[level].cell_masks.empty()) return nullptr;
  return g->lev[level].cell_masks.data();
}
int gen_kind(const gmg_gen *g) { return g ? g->kind : -1; }
}  // namespace gmg

extern "C" {

int gmg_gen_create(int kind, int nref, unsigned long long seed, double corr, double var, gmg_gen **out) {
  if (!out || kind < 0 || kind > 3 || nref < 0 || nref > (kind == 1 ? 9 : kind == 3 ? 7 : 12)) {
    gmg::set_error("gmg_gen_create: bad arguments (kind %d, nref %d)", kind, nref);
    return 1;
  }
  auto G = std::make_unique<gmg_gen>();
  G->kind = kind;
  G->nref = nref;
  G->lev.resize(nref + 1);
  const int dim = kind == 1 || kind == 3 ? 3 : 2;
  ugfx::LogNormalField field;
  if (var > 0.0 && kind != 2) field = ugfx::LogNormalField(seed, dim, corr, var);
  if (kind == 3) {
    if (build_ug_cube(G.get(), field)) return 1;
  } else {
    for (int l = 0; l <= nref; ++l)
      if (build_level(G.get(), l, field)) return 1;
  }
  G->desc.resize(nref + 1);
  for (int l = 0; l <= nref; ++l) {
    GenLevel &L = G->lev[l];
    gmg_level_desc &d = G->desc[l];
    d.n = L.n; d.s = L.s;
    d.rowptr = L.rowptr.data(); d.col = L.col.data(); d.val = L.val.data();
    d.vclass = L.vclass.data(); d.vnclass = L.vnclass.data(); d.skip = L.skip.data();
    d.prowptr = l ? L.prow.data() : nullptr;
    d.pcol = l ? L.pcol.data() : nullptr;
    d.pw = l ? L.pw.data() : nullptr;
  }
  // right-hand side on the finest level
  GenLevel &T = G->lev[nref];
  const int s = T.s;
  const double scale = double(1 << nref), hd = std::pow(1.0 / scale, dim);
  G->rhs.assign(size_t(T.n) * s, 0.0);
  for (int r = 0; r < T.n; ++r) {
    const double *x = &T.xyz[size_t(r) * 3];
    uint64_t key = ugfx::lattice_key(llround(x[0] * scale), llround(x[1] * scale), dim == 3 ? llround(x[2] * scale) : 0);
    for (int c = 0; c < s; ++c)
      G->rhs[size_t(r) * s + c] = (T.skip[r] & (1 << c)) ? 0.0 : ugfx::rhs_uniform(seed + 0x9E37ull * c, key) * hd;
  }
  *out = G.release();
  return 0;
}

int gmg_gen_levels(gmg_gen *g, const gmg_level_desc **levels, int *nlevels) {
  if (!g || !levels || !nlevels) return 1;
  *levels = g->desc.data();
  *nlevels = int(g->desc.size());
  return 0;
}

int gmg_gen_rhs(gmg_gen *g, const double **rhs, int *len) {
  if (!g || !rhs || !len) return 1;
  *rhs = g->rhs.data();
  *len = int(g->rhs.size());
  return 0;
}

int gmg_gen_coords(gmg_gen *g, int level, const double **xyz) {
  if (!g || !xyz || level < 0 || level >= int(g->lev.size())) return 1;
  *xyz = g->lev[level].xyz.data();
  return 0;
}

int gmg_gen_destroy(gmg_gen *g) {
  delete g;
  return 0;
}

}  // extern "C"
