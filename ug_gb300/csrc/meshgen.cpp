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

extern "C" {

int gmg_gen_create(int kind, int nref, unsigned long long seed, double corr, double var, gmg_gen **out) {
  if (!out || kind < 0 || kind > 2 || nref < 0 || nref > (kind == 1 ? 9 : 12)) {
    gmg::set_error("gmg_gen_create: bad arguments (kind %d, nref %d)", kind, nref);
    return 1;
  }
  auto G = std::make_unique<gmg_gen>();
  G->kind = kind;
  G->nref = nref;
  G->lev.resize(nref + 1);
  const int dim = kind == 1 ? 3 : 2;
  ugfx::LogNormalField field;
  if (var > 0.0 && kind != 2) field = ugfx::LogNormalField(seed, dim, corr, var);
  for (int l = 0; l <= nref; ++l)
    if (build_level(G.get(), l, field)) return 1;
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
