// ug_export: drives the UG 3.12.1 reference library (built from its own
// sources by oracle/Makefile) to produce golden data for the lmgc hot path.
// TEST ORACLE ONLY -- the ug_gb300 product never links or runs this.
//
// It builds a multigrid hierarchy with UG's own grid manager (coarse grid,
// `mark $a; refine` L times), assembles one system per level with the
// element rules below, and writes, in a small named-array container:
//   * the hierarchy exactly as UG stores it: per level the VECTOR list order,
//     each row's MATRIX list (diagonal first, VSTART/MNEXT order), the
//     VCLASS / VNCLASS / VECSKIP fields and node coordinates, and the
//     standard-transfer weights (corner -> father copy, otherwise the father
//     element's shape functions GNs at LCVECT, transgrid.cc:117-232);
//   * known-answer vectors of UG's kernels on the finest level:
//     dmatmul_minus (ugblas.cc:3997), l_jac (ugiter.cc:271), l_lgs
//     (ugiter.cc:412), l_ilubthdecomp + l_luiter (ugiter.cc:2252, 4444),
//     StandardRestrict / StandardInterpolateCorrection (transgrid.cc:462, 529),
//     dnrm2x (ugblas.cc:3156);
//   * a full `ls` + `lmgc` solve through UG's numproc interface
//     (NP_LINEAR_SOLVER, ls.cc:637): iteration count, first/last defect and
//     the final solution, plus the per-iteration defect history obtained by
//     replaying the ls loop (dset, Lmgc, dadd, dnrm2x) through the same
//     numprocs;
//   * the same problem solved with UG's cg and bcgs (ls.cc:901, 1711)
//     preconditioned by the same lmgc: iterations, defects, solution;
//   * with imat = block: an interpolation matrix (IMATRIX, VISTART lists) on
//     every fine level, the standard transfer's weights times a seeded block
//     near the identity, its known-answer vectors of RestrictByMatrix and
//     InterpolateCorrectionByMatrix (transgrid.cc:1113, 1292), and every
//     solve above with the transfer in its matrix mode (`$M`).
//
// usage: ug_export{2d,3d} <problem> <nref> <baselevel> <smoother> <seed> <out>
//        [maxit] [local_levels] [order] [imat]
//   problem  : poisson  (2D: one Q1 quad; 3D: six Kuhn tets of the unit cube)
//              diffusion (3D only: P1 with k = exp(g) per element, corr 0.1, var 1)
//              elasticity (2D only: P1 triangles, plane strain E=1 nu=0.3, 2x2 blocks)
//              lshape (2D only: the same elasticity on the L-shaped domain
//                (-1,1)^2 minus [0,1)x(-1,0], six coarse triangles; <nref>
//                uniform refinements, then <local_levels> local ones: step k
//                marks every leaf element with a corner within 0.5^k of the
//                re-entrant corner for red refinement, UG closes the grid
//                (green closure, yellow copies); the right-hand side lives on
//                the surface vectors of every level)
//   smoother : jac (damp 0.8) | gs | ilu
#include <config.h>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <chrono>
#include <string>
#include <unordered_map>
#include <vector>

#include "cmdint.h"
#include "commands.h"
#include "gm.h"
#include "initug.h"
#include "iter.h"
#include "ls.h"
#include "np.h"
#include "numproc.h"
#include "order.h"
#include "shapes.h"
#include "std_domain.h"
#include "transfer.h"
#include "udm.h"
#include "ugdevices.h"
#include "ugm.h"

#include "../ug_gb300/csrc/fields.h"

USING_UG_NAMESPACES

#ifdef _2
static const int DIMX = 2;
#else
static const int DIMX = 3;
#endif

// ---------------------------------------------------------------- container
// "UGFX1\n" then records: name\0, type char ('d' f64, 'i' i32, 's' bytes), int64 count, data
static FILE *g_out = nullptr;
static void put(const std::string &name, char t, const void *p, int64_t n) {
  fwrite(name.c_str(), 1, name.size() + 1, g_out);
  fwrite(&t, 1, 1, g_out);
  fwrite(&n, sizeof(n), 1, g_out);
  size_t es = (t == 'd' || t == 'q') ? 8 : (t == 's' ? 1 : 4);
  if (n) fwrite(p, es, size_t(n), g_out);
}
static void putd(const std::string &n, const std::vector<double> &v) { put(n, 'd', v.data(), (int64_t)v.size()); }
static void puti(const std::string &n, const std::vector<int> &v) { put(n, 'i', v.data(), (int64_t)v.size()); }
static void put1(const std::string &n, double x) { put(n, 'd', &x, 1); }
static void put1i(const std::string &n, int x) { put(n, 'i', &x, 1); }

static INT BndCond(void *, void *, DOUBLE *, DOUBLE *value, INT *type) { value[0] = 0.0; type[0] = 0; return 0; }

// the L-shaped domain: eight corners counter-clockwise (the long edges split
// so that the six coarse triangles use corners only), straight segments
static double g_lcorner[8][2] = {{-1, -1}, {0, -1}, {0, 0}, {1, 0}, {1, 1}, {0, 1}, {-1, 1}, {-1, 0}};
static double g_lseg[8][4];
static INT lshape_segment(void *data, DOUBLE *param, DOUBLE *result) {
  const double *e = (const double *)data, t = param[0];
  if (t < 0.0 || t > 1.0) return 1;
  result[0] = (1.0 - t) * e[0] + t * e[2];
  result[1] = (1.0 - t) * e[1] + t * e[3];
  return 0;
}
static int create_lshape_domain() {
  DOUBLE mid[2] = {0.0, 0.0};
  if (!CreateDomain("LShape", mid, 1.5, 8, 8, NO)) return 1;
  for (int i = 0; i < 8; ++i) {
    const int j = (i + 1) % 8;
    g_lseg[i][0] = g_lcorner[i][0]; g_lseg[i][1] = g_lcorner[i][1];
    g_lseg[i][2] = g_lcorner[j][0]; g_lseg[i][3] = g_lcorner[j][1];
    char name[16];
    snprintf(name, sizeof name, "side%d", i);
    if (!CreateBoundarySegment2D(name, 1, 0, i, i, j, 1, 0.0, 1.0, lshape_segment, g_lseg[i])) return 1;
  }
  return 0;
}
static void run(const char *c) {
  char b[4096];
  snprintf(b, sizeof b, "%s", c);
  INT e = InterpretCommand(b);
  if (e) { fprintf(stderr, "UG command failed (%d): %s\n", (int)e, c); exit(1); }
}

// per-level vector numbering in list order (independent of VINDEX)
struct LevelIndex {
  std::unordered_map<const VECTOR *, int> idx;
  std::vector<VECTOR *> vecs;
};
static std::vector<LevelIndex> g_lev;

static void index_levels(MULTIGRID *mg) {
  g_lev.assign(TOPLEVEL(mg) + 1, LevelIndex());
  for (int l = 0; l <= TOPLEVEL(mg); ++l)
    for (VECTOR *v = FIRSTVECTOR(GRID_ON_LEVEL(mg, l)); v; v = SUCCVC(v)) {
      g_lev[l].idx[v] = (int)g_lev[l].vecs.size();
      g_lev[l].vecs.push_back(v);
    }
}

static const double *node_xyz(NODE *n) { return CVECT(MYVERTEX(n)); }

// ------------------------------------------------------------------ assembly
// 2D Q1 Laplacian on the (square) element: K/6 with the classic stencil.
static const double KQ1[4][4] = {{4, -1, -2, -1}, {-1, 4, -1, -2}, {-2, -1, 4, -1}, {-1, -2, -1, 4}};

// P1 simplex gradients: G[i][d] = d(phi_i)/dx_d, returns |det J|
static double p1_grads(int dim, double X[4][3], double G[4][3]) {
  if (dim == 2) {
    double J00 = X[1][0] - X[0][0], J01 = X[2][0] - X[0][0];
    double J10 = X[1][1] - X[0][1], J11 = X[2][1] - X[0][1];
    double det = J00 * J11 - J01 * J10;
    double i00 = J11 / det, i01 = -J01 / det, i10 = -J10 / det, i11 = J00 / det;
    // rows of J^{-1} are gradients of the reference barycentrics 1,2
    G[1][0] = i00; G[1][1] = i01; G[2][0] = i10; G[2][1] = i11;
    G[0][0] = -(i00 + i10); G[0][1] = -(i01 + i11);
    return std::fabs(det);
  }
  double J[3][3];
  for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) J[r][c] = X[c + 1][r] - X[0][r];
  double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
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
  return std::fabs(det);
}

static MATRIX *mat_of(VECTOR *a, VECTOR *b) {
  MATRIX *m = (a == b) ? VSTART(a) : GetMatrix(a, b);
  if (!m) { fprintf(stderr, "missing matrix connection\n"); exit(1); }
  return m;
}

int main(int argc, char **argv) {
  if (argc < 7) {
    fprintf(stderr, "usage: %s problem nref baselevel smoother seed out [maxit] [nloc] [order]\n", argv[0]);
    return 2;
  }
  std::string problem = argv[1];
  int nref = atoi(argv[2]), baselevel = atoi(argv[3]);
  std::string smoother = argv[4];
  uint64_t seed = strtoull(argv[5], nullptr, 10);
  const char *outfile = argv[6];
  int maxit = argc > 7 ? atoi(argv[7]) : 100;
  int nloc = argc > 8 ? atoi(argv[8]) : 0;
  // UG's ordering numprocs (order.cc:931) applied to every level after the
  // assembly: "bw" (order.bw) or "lex:<config>" (order.lex $config <config>)
  std::string order = argc > 9 ? argv[9] : "none";
  // "block": IMATRIX on every fine level and the transfer in `$M` mode
  const bool imat = argc > 10 && std::string(argv[10]) == "block";
  char cmd[512];
  int ug_argc = 1;
  char *ug_argv0 = argv[0];
  char **ug_argv = &ug_argv0;
  if (InitUg(&ug_argc, &ug_argv)) return 1;

  const bool lshape = problem == "lshape";
  const bool elast = problem == "elasticity" || lshape;
  const bool diffusion = problem == "diffusion";
  if ((elast && DIMX != 2) || (diffusion && DIMX != 3)) { fprintf(stderr, "problem/dimension mismatch\n"); return 2; }
  if (nloc > 0 && !lshape) { fprintf(stderr, "local refinement is defined for lshape only\n"); return 2; }
  const int s = elast ? 2 : 1;

  CreateBoundaryValueProblem("bvp", BndCond, 0, NULL, 0, NULL);
  if (lshape && create_lshape_domain()) { fprintf(stderr, "L-shaped domain\n"); return 1; }
  run(lshape ? "configure bvp $d LShape;" : DIMX == 2 ? "configure bvp $d Quadrilateral;" : "configure bvp $d Hexahedron;");
  if (imat) run(s == 1 ? "newformat fmt $V n1: vt 20 $M implicit(vt): mt 4 $I n1;"
                       : "newformat fmt $V n2: vt 20 $M implicit(vt): mt 4 $I n2;");
  else run(s == 1 ? "newformat fmt $V n1: vt 20 $M implicit(vt): mt 4;" : "newformat fmt $V n2: vt 20 $M implicit(vt): mt 4;");
  run("new mg $b bvp $f fmt $h 4000M;");
  if (lshape) {
    // three unit squares, each split by its diagonal through the re-entrant corner (node 2)
    run("ie 0 1 2;"); run("ie 0 2 7;"); run("ie 7 2 6;"); run("ie 2 5 6;"); run("ie 2 3 4;"); run("ie 2 4 5;");
  } else if (DIMX == 2 && !elast) run("ie 0 1 2 3;");
  else if (DIMX == 2) { run("ie 0 1 2;"); run("ie 0 2 3;"); }
  else { run("ie 0 1 2 6;"); run("ie 0 2 3 6;"); run("ie 0 3 7 6;"); run("ie 0 7 4 6;"); run("ie 0 4 5 6;"); run("ie 0 5 1 6;"); }
  run("fixcoarsegrid;");
  for (int l = 0; l < nref; ++l) { run("mark $a;"); run("refine;"); }
  for (int k = 1; k <= nloc; ++k) {
    // mark the leaf elements near the re-entrant corner (0, 0); refine closes the grid
    MULTIGRID *m0 = GetCurrentMultigrid();
    const double r = std::ldexp(1.0, -k);
    int nmarked = 0;
    for (int l = 0; l <= TOPLEVEL(m0); ++l)
      for (ELEMENT *e = FIRSTELEMENT(GRID_ON_LEVEL(m0, l)); e; e = SUCCE(e)) {
        if (!EstimateHere(e)) continue;
        bool near = false;
        for (int i = 0; i < CORNERS_OF_ELEM(e); ++i) {
          const double *x = node_xyz(CORNER(e, i));
          if (x[0] * x[0] + x[1] * x[1] <= r * r) near = true;
        }
        if (near) { if (MarkForRefinement(e, RED, 0)) { fprintf(stderr, "mark failed\n"); return 1; } ++nmarked; }
      }
    fprintf(stderr, "local step %d: %d elements marked\n", k, nmarked);
    run("refine;");
  }
  run("createvector sol rhs kx ky kd kv kc kt;");
  run("creatematrix MAT LU;");

  MULTIGRID *mg = GetCurrentMultigrid();
  const int top = TOPLEVEL(mg);
  VECDATA_DESC *sol = GetVecDataDescByName(mg, (char *)"sol"), *rhs = GetVecDataDescByName(mg, (char *)"rhs");
  VECDATA_DESC *kx = GetVecDataDescByName(mg, (char *)"kx"), *ky = GetVecDataDescByName(mg, (char *)"ky");
  VECDATA_DESC *kd = GetVecDataDescByName(mg, (char *)"kd"), *kv = GetVecDataDescByName(mg, (char *)"kv");
  VECDATA_DESC *kc = GetVecDataDescByName(mg, (char *)"kc"), *kt = GetVecDataDescByName(mg, (char *)"kt");
  MATDATA_DESC *A = GetMatDataDescByName(mg, (char *)"MAT"), *LU = GetMatDataDescByName(mg, (char *)"LU");
  const SHORT *mcmp = MD_MCMPPTR_OF_RT_CT(A, NODEVEC, NODEVEC);
  const SHORT *lucmp = MD_MCMPPTR_OF_RT_CT(LU, NODEVEC, NODEVEC);
  auto vcmp = [](VECDATA_DESC *vd) { return VD_CMPPTR_OF_TYPE(vd, NODEVEC); };

  ugfx::LogNormalField field;
  if (diffusion) field = ugfx::LogNormalField(seed, 3, 0.1, 1.0);
  const double nu = 0.3, E = 1.0;
  const double lam = E * nu / ((1 + nu) * (1 - 2 * nu)), mu = E / (2 * (1 + nu));

  // ---- assemble every level
  for (int l = 0; l <= top; ++l) {
    GRID *g = GRID_ON_LEVEL(mg, l);
    for (VECTOR *v = FIRSTVECTOR(g); v; v = SUCCVC(v)) {
      for (int c = 0; c < s; ++c) { VVALUE(v, vcmp(sol)[c]) = 0; VVALUE(v, vcmp(rhs)[c]) = 0; }
      VECSKIP(v) = 0;
      for (MATRIX *m = VSTART(v); m; m = MNEXT(m)) for (int k = 0; k < s * s; ++k) MVALUE(m, mcmp[k]) = 0;
    }
    for (ELEMENT *e = FIRSTELEMENT(g); e; e = SUCCE(e)) {
      int nc = CORNERS_OF_ELEM(e);
      VECTOR *vv[8];
      double X[8][3] = {{0}};
      for (int i = 0; i < nc; ++i) {
        vv[i] = NVECTOR(CORNER(e, i));
        for (int d = 0; d < DIMX; ++d) X[i][d] = node_xyz(CORNER(e, i))[d];
      }
      if (DIMX == 2 && nc == 4) {
        for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) MVALUE(mat_of(vv[i], vv[j]), mcmp[0]) += KQ1[i][j] / 6.0;
      } else if (!elast) {
        double G[4][3] = {{0}};
        double det = p1_grads(DIMX, X, G);
        double vol = det / (DIMX == 2 ? 2.0 : 6.0);
        double kk = 1.0;
        if (diffusion) {
          double xc[3] = {0, 0, 0};
          for (int i = 0; i < nc; ++i) for (int d = 0; d < 3; ++d) xc[d] += X[i][d] / nc;
          kk = field.k(xc);
        }
        for (int i = 0; i < nc; ++i)
          for (int j = 0; j < nc; ++j) {
            double a = 0;
            for (int d = 0; d < DIMX; ++d) a += G[i][d] * G[j][d];
            MVALUE(mat_of(vv[i], vv[j]), mcmp[0]) += kk * vol * a;
          }
      } else {
        // plane strain: K_ij(a,b) = area * (lam dphi_i/da dphi_j/db + mu dphi_i/db dphi_j/da + mu delta_ab grad.grad)
        double G[4][3] = {{0}};
        double area = p1_grads(2, X, G) / 2.0;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            MATRIX *m = mat_of(vv[i], vv[j]);
            double gg = G[i][0] * G[j][0] + G[i][1] * G[j][1];
            for (int a = 0; a < 2; ++a)
              for (int b = 0; b < 2; ++b)
                MVALUE(m, mcmp[a * 2 + b]) += area * (lam * G[i][a] * G[j][b] + mu * G[i][b] * G[j][a] + (a == b ? mu * gg : 0.0));
          }
      }
    }
    // homogeneous Dirichlet on the whole boundary: unit row, VECSKIP on all components
    for (NODE *n = FIRSTNODE(g); n; n = SUCCN(n))
      if (OBJT(MYVERTEX(n)) == BVOBJ) VECSKIP(NVECTOR(n)) = (1 << s) - 1;
    for (VECTOR *v = FIRSTVECTOR(g); v; v = SUCCVC(v))
      if (VECSKIP(v)) {
        MATRIX *m = VSTART(v);
        for (int k = 0; k < s * s; ++k) MVALUE(m, mcmp[k]) = (k % (s + 1) == 0) ? 1.0 : 0.0;
        for (m = MNEXT(m); m; m = MNEXT(m)) for (int k = 0; k < s * s; ++k) MVALUE(m, mcmp[k]) = 0.0;
      }
  }
  // ---- seeded right-hand side, keyed by lattice position
  if (lshape) {
    // on the surface: FINE_GRID_DOF vectors below the top level, NEW_DEFECT
    // vectors on it (the rows UG's ON_SURFACE loops visit, np/algebra/vecloop.ct);
    // a surface vector on level l carries f * h_l^2 with h_l = 2^-l
    const double scale = std::ldexp(1.0, top);
    for (int l = 0; l <= top; ++l) {
      const double hd = std::ldexp(1.0, -2 * l);
      for (NODE *n = FIRSTNODE(GRID_ON_LEVEL(mg, l)); n; n = SUCCN(n)) {
        VECTOR *v = NVECTOR(n);
        if (!(l == top ? NEW_DEFECT(v) : FINE_GRID_DOF(v))) continue;
        const double *x = node_xyz(n);
        int64_t ix = llround((x[0] + 1.0) * scale), iy = llround((x[1] + 1.0) * scale);
        uint64_t key = ugfx::lattice_key(ix, iy, 0);
        for (int c = 0; c < s; ++c)
          VVALUE(v, vcmp(rhs)[c]) = (VECSKIP(v) & (1 << c)) ? 0.0 : ugfx::rhs_uniform(seed + 0x9E37ull * c, key) * hd;
      }
    }
  } else {
    const double scale = double(1 << nref);
    const double hd = std::pow(1.0 / scale, DIMX);
    for (NODE *n = FIRSTNODE(GRID_ON_LEVEL(mg, top)); n; n = SUCCN(n)) {
      VECTOR *v = NVECTOR(n);
      const double *x = node_xyz(n);
      int64_t ix = llround(x[0] * scale), iy = llround(x[1] * scale), iz = DIMX == 3 ? llround(x[2] * scale) : 0;
      uint64_t key = ugfx::lattice_key(ix, iy, iz);
      for (int c = 0; c < s; ++c)
        VVALUE(v, vcmp(rhs)[c]) = (VECSKIP(v) & (1 << c)) ? 0.0 : ugfx::rhs_uniform(seed + 0x9E37ull * c, key) * hd;
    }
  }

  if (order != "none") {
    if (order == "bw") {
      run("npcreate ord $c bw; npinit ord;");
    } else if (order.compare(0, 4, "lex:") == 0) {
      snprintf(cmd, sizeof cmd, "npcreate ord $c lex; npinit ord $config %s;", order.c_str() + 4);
      run(cmd);
    } else {
      fprintf(stderr, "unknown order %s\n", order.c_str());
      return 2;
    }
    NP_ORDER *ord = (NP_ORDER *)GetNumProcByName(mg, "ord", ORDER_CLASS_NAME);
    if (!ord) { fprintf(stderr, "no order numproc\n"); return 1; }
    for (int l = 0; l <= top; ++l) {
      INT res = 0;
      if ((*ord->Order)(ord, l, NULL, &res)) { fprintf(stderr, "order failed on level %d\n", l); return 1; }
    }
  }
  index_levels(mg);
  for (int l = 0; l <= top; ++l) {  // element census per level: corners, refinement class
    int cnt[5][4] = {{0}};
    for (ELEMENT *e = FIRSTELEMENT(GRID_ON_LEVEL(mg, l)); e; e = SUCCE(e)) cnt[CORNERS_OF_ELEM(e)][ECLASS(e)]++;
    fprintf(stderr, "level %d elements: tri yellow/green/red %d/%d/%d quad %d\n", l, cnt[3][YELLOW_CLASS],
            cnt[3][GREEN_CLASS], cnt[3][RED_CLASS], cnt[4][0] + cnt[4][1] + cnt[4][2] + cnt[4][3]);
  }
  g_out = fopen(outfile, "wb");
  if (!g_out) { perror(outfile); return 1; }
  fwrite("UGFX1\n", 1, 6, g_out);
  put1i("dim", DIMX); put1i("nlevels", top + 1); put1i("baselevel", baselevel); put1i("blocksize", s);
  put1i("nref", nref); put1i("seed", (int)seed); put1i("nloc", nloc);
  put1i("fullrefinelevel", FULLREFINELEVEL(mg));
  put("problem", 's', problem.c_str(), (int64_t)problem.size());
  put("smoother", 's', smoother.c_str(), (int64_t)smoother.size());
  put("order", 's', order.c_str(), (int64_t)order.size());

  // ---- hierarchy
  for (int l = 0; l <= top; ++l) {
    auto &L = g_lev[l];
    const int n = (int)L.vecs.size();
    std::vector<int> rowptr(1, 0), col, vclass(n), vnclass(n), skip(n);
    std::vector<double> val, xyz(size_t(n) * 3, 0.0);
    for (int i = 0; i < n; ++i) {
      VECTOR *v = L.vecs[i];
      vclass[i] = VCLASS(v); vnclass[i] = VNCLASS(v); skip[i] = VECSKIP(v);
      NODE *nd = (NODE *)VOBJECT(v);
      for (int d = 0; d < DIMX; ++d) xyz[size_t(i) * 3 + d] = node_xyz(nd)[d];
      for (MATRIX *m = VSTART(v); m; m = MNEXT(m)) {
        col.push_back(L.idx.at(MDEST(m)));
        for (int k = 0; k < s * s; ++k) val.push_back(MVALUE(m, mcmp[k]));
      }
      rowptr.push_back((int)col.size());
    }
    std::string p = "L" + std::to_string(l) + "_";
    put1i(p + "n", n); puti(p + "rowptr", rowptr); puti(p + "col", col); putd(p + "val", val);
    puti(p + "vclass", vclass); puti(p + "vnclass", vnclass); puti(p + "skip", skip); putd(p + "xyz", xyz);
    {
      std::vector<int> fg(n), nd(n);
      for (int i = 0; i < n; ++i) { fg[i] = FINE_GRID_DOF(L.vecs[i]) ? 1 : 0; nd[i] = NEW_DEFECT(L.vecs[i]) ? 1 : 0; }
      puti(p + "fine_grid_dof", fg); puti(p + "new_defect", nd);
    }
    if (l == 0) continue;
    // standard transfer weights, one row per fine vector
    std::vector<std::vector<std::pair<int, double>>> prow(n);
    for (NODE *nd = FIRSTNODE(GRID_ON_LEVEL(mg, l)); nd; nd = SUCCN(nd)) {
      int fi = L.idx.at(NVECTOR(nd));
      if (CORNERTYPE(nd)) {
        prow[fi].push_back({g_lev[l - 1].idx.at(NVECTOR((NODE *)NFATHER(nd))), 1.0});
      } else {
        VERTEX *vx = MYVERTEX(nd);
        ELEMENT *fe = VFATHER(vx);
        int nc = CORNERS_OF_ELEM(fe);
        DOUBLE c[MAX_CORNERS_OF_ELEM];
        GNs(nc, LCVECT(vx), c);
        for (int i = 0; i < nc; ++i)
          if (c[i] != 0.0) prow[fi].push_back({g_lev[l - 1].idx.at(NVECTOR(CORNER(fe, i))), c[i]});
      }
    }
    std::vector<int> pptr(1, 0), pcol;
    std::vector<double> pw;
    for (int i = 0; i < n; ++i) {
      for (auto &e : prow[i]) { pcol.push_back(e.first); pw.push_back(e.second); }
      pptr.push_back((int)pcol.size());
    }
    std::string q = "P" + std::to_string(l) + "_";
    puti(q + "rowptr", pptr); puti(q + "col", pcol); putd(q + "w", pw);
  }
  {
    std::vector<double> b, ball;
    for (VECTOR *v : g_lev[top].vecs) for (int c = 0; c < s; ++c) b.push_back(VVALUE(v, vcmp(rhs)[c]));
    putd("rhs", b);
    for (int l = 0; l <= top; ++l)
      for (VECTOR *v : g_lev[l].vecs) for (int c = 0; c < s; ++c) ball.push_back(VVALUE(v, vcmp(rhs)[c]));
    putd("rhs_all", ball);  // every level, levels concatenated
  }

  // ---- interpolation matrices (IMATRIX): for every fine vector and every
  // coarse vector of its standard transfer row (weight c), the block
  // c (I + 0.2 (U - 1/2)), U uniform[0,1) per entry from a seeded sequence
  // (coarse-component-major, as MVALUE of an interpolation matrix); exported
  // per level in VISTART order
  if (imat) {
    ugfx::SplitMix irng(seed * 104729 + 3);
    for (int l = 1; l <= top; ++l) {
      GRID *g = GRID_ON_LEVEL(mg, l);
      for (NODE *nd = FIRSTNODE(g); nd; nd = SUCCN(nd)) {
        VECTOR *v = NVECTOR(nd);
        std::vector<std::pair<VECTOR *, double>> row;
        if (CORNERTYPE(nd)) {
          row.push_back({NVECTOR((NODE *)NFATHER(nd)), 1.0});
        } else {
          VERTEX *vx = MYVERTEX(nd);
          ELEMENT *fe = VFATHER(vx);
          int nc = CORNERS_OF_ELEM(fe);
          DOUBLE c[MAX_CORNERS_OF_ELEM];
          GNs(nc, LCVECT(vx), c);
          for (int i = 0; i < nc; ++i)
            if (c[i] != 0.0) row.push_back({NVECTOR(CORNER(fe, i)), c[i]});
        }
        for (auto &e : row) {
          MATRIX *im = CreateIMatrix(g, v, e.first);
          if (!im) { fprintf(stderr, "CreateIMatrix failed\n"); return 1; }
          for (int i = 0; i < s; ++i)
            for (int j = 0; j < s; ++j)
              MVALUEPTR(im, 0)[i * s + j] = e.second * ((i == j ? 1.0 : 0.0) + 0.2 * (irng.uniform() - 0.5));
        }
      }
      auto &L = g_lev[l];
      std::vector<int> mptr(1, 0), mcol;
      std::vector<double> mval;
      for (VECTOR *v : L.vecs) {
        for (MATRIX *im = VISTART(v); im; im = MNEXT(im)) {
          mcol.push_back(g_lev[l - 1].idx.at(MDEST(im)));
          for (int k = 0; k < s * s; ++k) mval.push_back(MVALUEPTR(im, 0)[k]);
        }
        mptr.push_back((int)mcol.size());
      }
      std::string q = "M" + std::to_string(l) + "_";
      puti(q + "rowptr", mptr); puti(q + "col", mcol); putd(q + "val", mval);
    }
  }
  put1i("imat", imat ? 1 : 0);

  // ---- kernel known-answer vectors on the finest level
  ugfx::SplitMix rng(seed * 7919 + 17);
  GRID *gt = GRID_ON_LEVEL(mg, top);
  GRID *gc = GRID_ON_LEVEL(mg, top - 1);
  auto fill = [&](VECDATA_DESC *vd, GRID *g) {
    for (VECTOR *v = FIRSTVECTOR(g); v; v = SUCCVC(v)) for (int c = 0; c < s; ++c) VVALUE(v, vcmp(vd)[c]) = 2 * rng.uniform() - 1;
  };
  auto grab = [&](VECDATA_DESC *vd, int l) {
    std::vector<double> r;
    for (VECTOR *v : g_lev[l].vecs) for (int c = 0; c < s; ++c) r.push_back(VVALUE(v, vcmp(vd)[c]));
    return r;
  };
  fill(kx, gt); fill(ky, gt); fill(kd, gt); fill(kv, gt);
  putd("kat_x", grab(kx, top)); putd("kat_y", grab(ky, top)); putd("kat_d", grab(kd, top));
  if (dmatmul_minus(mg, top, top, ALL_VECTORS, kx, A, ky)) return 1;
  putd("kat_matmul", grab(kx, top));
  if (l_jac(gt, kv, A, kd)) return 1;
  putd("kat_jac", grab(kv, top));
  fill(kv, gt);
  l_setindex(gt);
  if (l_lgs(gt, kv, A, kd, NULL)) return 1;
  putd("kat_gs", grab(kv, top));
  {
    VEC_SCALAR a;
    if (dnrm2x(mg, top, top, ALL_VECTORS, kd, a)) return 1;
    std::vector<double> nr(a, a + s);
    putd("kat_nrm", nr);
  }
  {
    if (dmatcopy(mg, top, top, ALL_VECTORS, LU, A)) return 1;
    VEC_SCALAR beta;
    for (int i = 0; i < MAX_VEC_COMP; ++i) beta[i] = 0.0;
    l_setindex(gt);
    if (l_ilubthdecomp(gt, LU, beta, NULL, NULL, NULL)) { fprintf(stderr, "ilu failed\n"); return 1; }
    std::vector<double> luv;
    for (VECTOR *v : g_lev[top].vecs)
      for (MATRIX *m = VSTART(v); m; m = MNEXT(m)) for (int k = 0; k < s * s; ++k) luv.push_back(MVALUE(m, lucmp[k]));
    putd("kat_ilu_factors", luv);
    fill(kv, gt);
    if (l_luiter(gt, kv, LU, kd)) return 1;
    putd("kat_ilu", grab(kv, top));
  }
  if (top >= 1) {
    VEC_SCALAR one;
    for (int i = 0; i < MAX_VEC_COMP; ++i) one[i] = 1.0;
    fill(kc, gc);
    putd("kat_restrict_pre", grab(kc, top - 1));
    if (StandardRestrict(gt, kc, kd, one)) return 1;
    putd("kat_restrict", grab(kc, top - 1));
    fill(kc, gc); fill(kt, gt);
    putd("kat_interp_coarse", grab(kc, top - 1));
    if (StandardInterpolateCorrection(gt, kt, kc, one)) return 1;
    putd("kat_interp", grab(kt, top));
    if (imat) {  // the matrix-mode transfers, plain and damped
      VEC_SCALAR dm;
      for (int i = 0; i < MAX_VEC_COMP; ++i) dm[i] = 0.7 - 0.1 * i;
      fill(kc, gc);
      putd("kat_mrestrict_pre", grab(kc, top - 1));
      if (RestrictByMatrix(gt, kc, kd, one)) return 1;
      putd("kat_mrestrict", grab(kc, top - 1));
      fill(kc, gc);
      putd("kat_mrestrict_damp_pre", grab(kc, top - 1));
      if (RestrictByMatrix(gt, kc, kd, dm)) return 1;
      putd("kat_mrestrict_damp", grab(kc, top - 1));
      fill(kc, gc); fill(kt, gt);
      putd("kat_minterp_coarse", grab(kc, top - 1));
      if (InterpolateCorrectionByMatrix(gt, kt, kc, one)) return 1;
      putd("kat_minterp", grab(kt, top));
      fill(kt, gt);
      if (InterpolateCorrectionByMatrix(gt, kt, kc, dm)) return 1;
      putd("kat_minterp_damp", grab(kt, top));
    }
  }

  // ---- full solve through UG's numprocs
  run(imat ? "npcreate transfer $c transfer; npinit transfer $M;" : "npcreate transfer $c transfer; npinit transfer;");
  // ---- the transfer numproc's solution operations on every level
  // (transfer.cc:775 InterpolateNewVectors -> StandardIntNewNodeVector,
  // transfer.cc:794 ProjectSolution -> StandardProject), with VNEW of the
  // last refinement step
  {
    NP_TRANSFER *tr = (NP_TRANSFER *)GetNumProcByName(mg, "transfer", TRANSFER_CLASS_NAME);
    if (!tr) { fprintf(stderr, "transfer lookup failed\n"); return 1; }
    auto grab_all = [&](VECDATA_DESC *vd) {
      std::vector<double> r;
      for (int l = 0; l <= top; ++l) { auto x = grab(vd, l); r.insert(r.end(), x.begin(), x.end()); }
      return r;
    };
    for (int l = 0; l <= top; ++l) {
      std::vector<int> vn;
      for (VECTOR *v : g_lev[l].vecs) vn.push_back(VNEW(v) ? 1 : 0);
      puti("L" + std::to_string(l) + "_vnew", vn);
    }
    for (int l = 0; l <= top; ++l) fill(kx, GRID_ON_LEVEL(mg, l));
    putd("kat_newvec_pre", grab_all(kx));
    INT r = 0;
    if ((*tr->InterpolateNewVectors)(tr, 0, top, kx, &r)) { fprintf(stderr, "InterpolateNewVectors failed\n"); return 1; }
    putd("kat_newvec", grab_all(kx));
    for (int l = 0; l <= top; ++l) fill(kx, GRID_ON_LEVEL(mg, l));
    putd("kat_project_pre", grab_all(kx));
    if ((*tr->ProjectSolution)(tr, 0, top, kx, &r)) { fprintf(stderr, "ProjectSolution failed\n"); return 1; }
    putd("kat_project", grab_all(kx));
  }
  if (smoother == "jac") run("npcreate smooth $c jac; npinit smooth $damp 0.8;");
  else if (smoother == "gs") run("npcreate smooth $c gs; npinit smooth;");
  else run("npcreate smooth $c ilu; npinit smooth;");
  run("npcreate base $c ex; npinit base;");
  run("npcreate basesolver $c ls; npinit basesolver $red 1e-14 $m 1 $I base;");
  snprintf(cmd, sizeof cmd, "npcreate lmgc $c lmgc; npinit lmgc $S smooth smooth basesolver $T transfer $n1 2 $n2 2 $b %d;", baselevel);
  run(cmd);
  snprintf(cmd, sizeof cmd, "npcreate mgs $c ls; npinit mgs $A MAT $x sol $b rhs $red 1e-10 $abslimit 1e-50 $m %d $I lmgc;", maxit);
  run(cmd);
  NP_LINEAR_SOLVER *ls = (NP_LINEAR_SOLVER *)GetNumProcByName(mg, "mgs", LINEAR_SOLVER_CLASS_NAME);
  NP_ITER *lmgc = (NP_ITER *)GetNumProcByName(mg, "lmgc", ITER_CLASS_NAME);
  if (!ls || !lmgc) { fprintf(stderr, "numproc lookup failed\n"); return 1; }
  // keep the rhs to replay the loop afterwards
  std::vector<std::vector<double>> rhs_lev;
  for (int l = 0; l <= top; ++l) rhs_lev.push_back(grab(rhs, l));
  auto restart = [&]() {  // x = 0 and the assembled right-hand side on every level
    for (int l = 0; l <= top; ++l) {
      dset(mg, l, l, ALL_VECTORS, sol, 0.0);
      size_t i = 0;
      for (VECTOR *v : g_lev[l].vecs) for (int c = 0; c < s; ++c) VVALUE(v, vcmp(rhs)[c]) = rhs_lev[l][i++];
    }
  };
  INT bl = 0, res = 0;
  LRESULT lr;
  memset(&lr, 0, sizeof lr);
  if ((*ls->PreProcess)(ls, top, sol, rhs, A, &bl, &res)) { fprintf(stderr, "PreProcess failed\n"); return 1; }
  (*ls->Defect)(ls, top, sol, rhs, A, &res);
  (*ls->Residuum)(ls, bl, top, sol, rhs, A, &lr);
  auto t0 = std::chrono::steady_clock::now();
  clock_t c0 = clock();
  if ((*ls->Solver)(ls, top, sol, rhs, A, ls->abslimit, ls->reduction, &lr)) { fprintf(stderr, "Solver failed\n"); return 1; }
  double cpu_s = double(clock() - c0) / CLOCKS_PER_SEC;
  double wall_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  put1i("ls_iters", lr.number_of_linear_iterations); put1i("ls_converged", lr.converged);
  putd("ls_first", std::vector<double>(lr.first_defect, lr.first_defect + s));
  putd("ls_last", std::vector<double>(lr.last_defect, lr.last_defect + s));
  putd("ls_x", grab(sol, top));
  {
    std::vector<double> xa;
    for (int l = 0; l <= top; ++l) { auto xl = grab(sol, l); xa.insert(xa.end(), xl.begin(), xl.end()); }
    putd("ls_x_all", xa);  // every level, levels concatenated (the surface solution spans levels)
  }
  put1("ls_wall_s", wall_s); put1("ls_cpu_s", cpu_s);
  fprintf(stderr, "UG ls: iters=%d converged=%d first=%.6e last=%.6e wall=%.3fs\n", (int)lr.number_of_linear_iterations,
          (int)lr.converged, lr.first_defect[0], lr.last_defect[0], wall_s);

  // replay: x = 0, b = rhs, then per iteration dset(c,0); Lmgc; x += c; |b|
  {
    restart();
    (*ls->Defect)(ls, top, sol, rhs, A, &res);
    std::vector<double> hist;
    VEC_SCALAR a;
    dnrm2x(mg, top, top, ON_SURFACE, rhs, a);
    for (int c = 0; c < s; ++c) hist.push_back(a[c]);
    int blv = baselevel < top ? baselevel : top;
    for (int it = 0; it < lr.number_of_linear_iterations; ++it) {
      dset(mg, top, top, ALL_VECTORS, kc, 0.0);
      if ((*lmgc->Iter)(lmgc, top, kc, rhs, A, &res)) { fprintf(stderr, "Lmgc failed\n"); return 1; }
      dadd(mg, blv, top, ALL_VECTORS, sol, kc);
      dnrm2x(mg, top, top, ON_SURFACE, rhs, a);
      for (int c = 0; c < s; ++c) hist.push_back(a[c]);
    }
    putd("ls_hist", hist);
    putd("ls_x_replay", grab(sol, top));
    // releases what the smoothers allocated (the ILU factor matrix)
    (*ls->PostProcess)(ls, top, sol, rhs, A, &res);
  }

  // ---- UG's cg (ls.cc:901-1165) preconditioned by the same lmgc, from x = 0
  {
    restart();
    snprintf(cmd, sizeof cmd, "npcreate cgs $c cg; npinit cgs $A MAT $x sol $b rhs $red 1e-10 $abslimit 1e-50 $m %d $I lmgc;",
             maxit);
    run(cmd);
    NP_LINEAR_SOLVER *cg = (NP_LINEAR_SOLVER *)GetNumProcByName(mg, "cgs", LINEAR_SOLVER_CLASS_NAME);
    if (!cg) { fprintf(stderr, "cg lookup failed\n"); return 1; }
    LRESULT lc;
    memset(&lc, 0, sizeof lc);
    if ((*cg->PreProcess)(cg, top, sol, rhs, A, &bl, &res)) { fprintf(stderr, "cg PreProcess failed\n"); return 1; }
    (*cg->Defect)(cg, top, sol, rhs, A, &res);
    (*cg->Residuum)(cg, bl, top, sol, rhs, A, &lc);
    if ((*cg->Solver)(cg, top, sol, rhs, A, cg->abslimit, cg->reduction, &lc)) {
      fprintf(stderr, "cg Solver failed\n");
      return 1;
    }
    put1i("cg_iters", lc.number_of_linear_iterations); put1i("cg_converged", lc.converged);
    putd("cg_first", std::vector<double>(lc.first_defect, lc.first_defect + s));
    putd("cg_last", std::vector<double>(lc.last_defect, lc.last_defect + s));
    putd("cg_x", grab(sol, top));
    {
      std::vector<double> xa;
      for (int l = 0; l <= top; ++l) { auto xl = grab(sol, l); xa.insert(xa.end(), xl.begin(), xl.end()); }
      putd("cg_x_all", xa);
    }
    fprintf(stderr, "UG cg: iters=%d converged=%d last=%.6e\n", (int)lc.number_of_linear_iterations, (int)lc.converged,
            lc.last_defect[0]);
    (*cg->PostProcess)(cg, top, sol, rhs, A, &res);
  }

  // ---- UG's bcgs (ls.cc:1711-2062) preconditioned by the same lmgc, from x = 0
  {
    restart();
    snprintf(cmd, sizeof cmd,
             "npcreate bcgs $c bcgs; npinit bcgs $A MAT $x sol $b rhs $red 1e-10 $abslimit 1e-50 $m %d $I lmgc;", maxit);
    run(cmd);
    NP_LINEAR_SOLVER *bs = (NP_LINEAR_SOLVER *)GetNumProcByName(mg, "bcgs", LINEAR_SOLVER_CLASS_NAME);
    if (!bs) { fprintf(stderr, "bcgs lookup failed\n"); return 1; }
    LRESULT lb;
    memset(&lb, 0, sizeof lb);
    if ((*bs->PreProcess)(bs, top, sol, rhs, A, &bl, &res)) { fprintf(stderr, "bcgs PreProcess failed\n"); return 1; }
    (*bs->Defect)(bs, top, sol, rhs, A, &res);
    (*bs->Residuum)(bs, bl, top, sol, rhs, A, &lb);
    if ((*bs->Solver)(bs, top, sol, rhs, A, bs->abslimit, bs->reduction, &lb)) {
      fprintf(stderr, "bcgs Solver failed\n");
      return 1;
    }
    put1i("bcgs_iters", lb.number_of_linear_iterations); put1i("bcgs_converged", lb.converged);
    putd("bcgs_first", std::vector<double>(lb.first_defect, lb.first_defect + s));
    putd("bcgs_last", std::vector<double>(lb.last_defect, lb.last_defect + s));
    putd("bcgs_x", grab(sol, top));
    {
      std::vector<double> xa;
      for (int l = 0; l <= top; ++l) { auto xl = grab(sol, l); xa.insert(xa.end(), xl.begin(), xl.end()); }
      putd("bcgs_x_all", xa);
    }
    fprintf(stderr, "UG bcgs: iters=%d converged=%d last=%.6e\n", (int)lb.number_of_linear_iterations,
            (int)lb.converged, lb.last_defect[0]);
  }
  (*ls->PostProcess)(ls, top, sol, rhs, A, &res);
  fclose(g_out);
  return 0;
}
