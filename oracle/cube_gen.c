/* cube_gen: the 3D diffusion workload's multigrid hierarchy, built without the
 * ug_gb300 library, for the oracle side of the tests and of the CPU baseline.
 *
 * TEST INFRASTRUCTURE ONLY (see lmgc_oracle.h): the product never calls it.
 *
 * Problem: -div(k grad u) = f on the unit cube, the six Kuhn tetrahedra
 * around the main diagonal (UG's coarse grid of the workload) red-refined
 * `nref` times, P1 elements assembled on every level, homogeneous Dirichlet
 * rows (unit diagonal, zero off-diagonals, VECSKIP) on the boundary, the
 * standard transfer weights of red refinement (corner copy 1, edge midpoint
 * 1/2 + 1/2; np/algebra/transgrid.cc:117-232 evaluated on these elements),
 * VCLASS 3 everywhere and VNCLASS 3 below the top level, 0 on it
 * (gm/algebra.cc:2838-2921 for a uniformly refined grid).
 *
 * Inputs are functions of position so that any grid manager that builds the
 * same mesh assembles the same system:
 *   k = exp(g) per tetrahedron, evaluated at its centroid, g a Gaussian field
 *   with exponential covariance var*exp(-r/corr) drawn by 256 random Fourier
 *   features (Rahimi & Recht 2007: frequencies from the multivariate Cauchy
 *   spectral density with scale 1/corr, phases uniform, amplitude
 *   sqrt(2 var / 256)); features drawn in sequence from splitmix64 (Steele,
 *   Lea & Flood 2014) seeded with mix(seed ^ 0x5eedf1e1d), normals by
 *   Box-Muller (cosine branch);
 *   f_i uniform[-1,1] keyed by the finest-level lattice position of node i
 *   and the seed, times h^3.
 * Node order on every level: lexicographic (x fastest).  Matrix rows: the
 * diagonal first, then the neighbours in the fixed lattice-offset order of
 * kOffs.  Element contributions are summed slab by slab (z layers of cells,
 * even layers first, then odd ones; in a layer y, x, then the six tetrahedra
 * of a cell), which fixes the rounding of every entry.
 *
 * Tetrahedra, rule 0: the Freudenthal triangulation of the lattice (cell
 * (i,j,k) split into the six tetrahedra x_s1 >= x_s2 >= x_s3 of its local
 * coordinates), which is what red refinement of the Kuhn tetrahedra gives
 * when every octahedron is cut along the diagonal that keeps that
 * triangulation.
 *
 * Rule 1: UG's own refinement.  The six coarse tetrahedra as the workload
 * inserts them (cube corners (0,1,2,6), (0,2,3,6), (0,3,7,6), (0,7,4,6),
 * (0,4,5,6), (0,5,1,6), cube corners numbered as UG's hexahedron domain
 * numbers them), refined by UG's red rules: the rule of the shortest
 * interior diagonal (ShortestInteriorEdge, gm/rm.cc:1567, its comparisons
 * and tie cases), the sons and their corner orders from UG's rule table
 * (TetrahedronRules, gm/rm.cc:494, rules 2-4: TET_RED_2_4, _0_5, _1_3,
 * gm/rm.h:183-186), edges numbered as UG numbers a tetrahedron's edges
 * (gm/elements.cc).  Every son lies in one lattice cell; rows list the
 * neighbours in the 26-direction order of kOffs26 (the 14 of rule 0 first),
 * elements are summed per z layer of cells (even layers, then odd), in a
 * layer by cell (y, x) and then by the sorted node numbers of the
 * element; a fine node off the coarse lattice interpolates from the ends of
 * the one coarse edge through it. */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "cube_gen.h"

/* ---- seeded inputs ------------------------------------------------------ */
static uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double u01(uint64_t z) { return (double)(z >> 11) * (1.0 / 9007199254740992.0); }
static uint64_t lattice_key(int64_t ix, int64_t iy, int64_t iz) {
  return ((uint64_t)ix << 42) ^ ((uint64_t)iy << 21) ^ (uint64_t)iz;
}
static double rhs_uniform(uint64_t seed, uint64_t key) { return 2.0 * u01(mix64(mix64(seed) ^ key)) - 1.0; }

typedef struct { uint64_t s; } sm_rng;
static uint64_t sm_next(sm_rng *r) { r->s += 0x9E3779B97F4A7C15ull; uint64_t z = r->s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull; z = (z ^ (z >> 27)) * 0x94D049BB133111EBull; return z ^ (z >> 31); }
static double sm_uniform(sm_rng *r) { return u01(sm_next(r)); }
static double sm_normal(sm_rng *r) {
  double u1 = sm_uniform(r), u2 = sm_uniform(r);
  if (u1 < 1e-300) u1 = 1e-300;
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

#define NFEAT 256
typedef struct { int on; double amp, w[NFEAT * 3], phi[NFEAT]; } field;

static void field_init(field *F, uint64_t seed, double corr, double var) {
  memset(F, 0, sizeof *F);
  if (!(var > 0.0)) return;
  sm_rng r = {mix64(seed ^ 0x5eedf1e1dull)};
  for (int m = 0; m < NFEAT; ++m) {
    double z0 = fabs(sm_normal(&r));
    if (z0 < 1e-12) z0 = 1e-12;
    for (int d = 0; d < 3; ++d) F->w[m * 3 + d] = sm_normal(&r) / (corr * z0);
    F->phi[m] = 6.283185307179586 * sm_uniform(&r);
  }
  F->amp = sqrt(2.0 * var / NFEAT);
  F->on = 1;
}

static double field_k(const field *F, const double *x) {
  if (!F->on) return 1.0;
  double s = 0.0;
  for (int m = 0; m < NFEAT; ++m) {
    double a = F->phi[m];
    for (int d = 0; d < 3; ++d) a += F->w[m * 3 + d] * x[d];
    s += cos(a);
  }
  return exp(F->amp * s);
}

/* ---- P1 element stiffness ----------------------------------------------- */
static void p1_stiffness(const double X[4][3], double kk, double *K) {
  double J[3][3], Ji[3][3], G[4][3];
  for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) J[r][c] = X[c + 1][r] - X[0][r];
  double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det; Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det; Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det; Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det; Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  for (int d = 0; d < 3; ++d) {
    G[1][d] = Ji[0][d]; G[2][d] = Ji[1][d]; G[3][d] = Ji[2][d];
    G[0][d] = -(Ji[0][d] + Ji[1][d] + Ji[2][d]);
  }
  const double vol = fabs(det) / 6.0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double a = 0;
      for (int d = 0; d < 3; ++d) a += G[i][d] * G[j][d];
      K[i * 4 + j] = kk * vol * a;
    }
}

/* ---- levels ------------------------------------------------------------- */
/* neighbour offsets in row order: for m = 1..7 (bits x, y, z) +m then -m */
static int kOffs[14][3];
static void init_offs(void) {
  int q = 0;
  for (int m = 1; m < 8; ++m) {
    int a = m & 1, b = (m >> 1) & 1, c = (m >> 2) & 1;
    kOffs[q][0] = a; kOffs[q][1] = b; kOffs[q][2] = c; ++q;
    kOffs[q][0] = -a; kOffs[q][1] = -b; kOffs[q][2] = -c; ++q;
  }
}

typedef struct {
  int n, N;
  int *rowptr, *col, *vclass, *vnclass, *skip, *prow, *pcol;
  double *val, *pw, *xyz;
} level;

struct orc_cube {
  int nref;
  level *lev;
  double *rhs;
  int rhs_len;
};

typedef struct { const field *F; double h; int N, t0, t1; double *kc; } field_job;
static const int kPerm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

/* corners of tetrahedron p of cell (i, j, t) */
static void tet_corners(int i, int j, int t, int p, int V[4][3]) {
  V[0][0] = i; V[0][1] = j; V[0][2] = t;
  for (int a = 1; a < 4; ++a) {
    for (int d = 0; d < 3; ++d) V[a][d] = V[a - 1][d];
    V[a][kPerm[p][a - 1]] += 1;
  }
}

/* k at the centroid of every tetrahedron of the slabs t0..t1-1 (index
 * ((t*nc + j)*nc + i)*6 + p) */
static void *field_slabs(void *arg) {
  field_job *J = (field_job *)arg;
  const int nc = J->N - 1;
  for (int t = J->t0; t < J->t1; ++t)
    for (int j = 0; j < nc; ++j)
      for (int i = 0; i < nc; ++i)
        for (int p = 0; p < 6; ++p) {
          int V[4][3];
          tet_corners(i, j, t, p, V);
          double xc[3] = {0, 0, 0};
          for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d) xc[d] += (V[a][d] * J->h) / 4;
          J->kc[(((size_t)t * nc + j) * nc + i) * 6 + p] = field_k(J->F, xc);
        }
  return NULL;
}

static int build_level(orc_cube *C, int l, const field *F, int nthreads) {
  level *L = &C->lev[l];
  const int N = (1 << l) + 1, n = N * N * N, nc = N - 1;
  const double h = 1.0 / (N - 1);
  L->N = N;
  L->n = n;
  L->rowptr = (int *)malloc(sizeof(int) * (n + 1));
  L->col = (int *)malloc(sizeof(int) * (size_t)n * 15);
  int *slot = (int *)malloc(sizeof(int) * (size_t)n * 14);
  L->xyz = (double *)malloc(sizeof(double) * (size_t)n * 3);
  if (!L->rowptr || !L->col || !slot || !L->xyz) return 1;
  int q = 0;
  L->rowptr[0] = 0;
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        int r = (k * N + j) * N + i;
        L->xyz[(size_t)r * 3] = i * h; L->xyz[(size_t)r * 3 + 1] = j * h; L->xyz[(size_t)r * 3 + 2] = k * h;
        L->col[q++] = r;
        for (int o = 0; o < 14; ++o) {
          int a = i + kOffs[o][0], b = j + kOffs[o][1], c = k + kOffs[o][2];
          slot[(size_t)r * 14 + o] = -1;
          if (a < 0 || b < 0 || c < 0 || a >= N || b >= N || c >= N) continue;
          slot[(size_t)r * 14 + o] = q;
          L->col[q++] = (c * N + b) * N + a;
        }
        L->rowptr[r + 1] = q;
      }
  L->val = (double *)calloc((size_t)q, sizeof(double));
  double *kc = (double *)malloc(sizeof(double) * ((size_t)nc * nc * nc * 6 + 1));
  if (!L->val || !kc) return 1;
  /* the field per element, slabs split over threads */
  int nt = nthreads < 1 ? 1 : nthreads;
  if (nt > nc) nt = nc > 0 ? nc : 1;
  pthread_t th[64];
  field_job jobs[64];
  if (nt > 64) nt = 64;
  for (int w = 0; w < nt; ++w) {
    jobs[w].F = F; jobs[w].h = h; jobs[w].N = N; jobs[w].kc = kc;
    jobs[w].t0 = (int)((long long)nc * w / nt); jobs[w].t1 = (int)((long long)nc * (w + 1) / nt);
  }
  for (int w = 1; w < nt; ++w) pthread_create(&th[w], NULL, field_slabs, &jobs[w]);
  if (nc > 0) field_slabs(&jobs[0]);
  for (int w = 1; w < nt; ++w) pthread_join(th[w], NULL);
  /* assembly: even slabs, then odd slabs */
  for (int parity = 0; parity < 2; ++parity)
    for (int t = parity; t < nc; t += 2)
      for (int j = 0; j < nc; ++j)
        for (int i = 0; i < nc; ++i)
          for (int p = 0; p < 6; ++p) {
            int V[4][3];
            double X[4][3], K[16];
            tet_corners(i, j, t, p, V);
            for (int a = 0; a < 4; ++a)
              for (int d = 0; d < 3; ++d) X[a][d] = V[a][d] * h;
            p1_stiffness(X, kc[(((size_t)t * nc + j) * nc + i) * 6 + p], K);
            for (int a = 0; a < 4; ++a) {
              int r = (V[a][2] * N + V[a][1]) * N + V[a][0];
              for (int b = 0; b < 4; ++b) {
                int e;
                if (a == b) {
                  e = L->rowptr[r];
                } else {
                  int dx = V[b][0] - V[a][0], dy = V[b][1] - V[a][1], dz = V[b][2] - V[a][2], o;
                  for (o = 0; o < 14; ++o)
                    if (kOffs[o][0] == dx && kOffs[o][1] == dy && kOffs[o][2] == dz) break;
                  e = slot[(size_t)r * 14 + o];
                }
                L->val[e] += K[a * 4 + b];
              }
            }
          }
  free(kc);
  free(slot);
  /* classes, Dirichlet rows */
  L->vclass = (int *)malloc(sizeof(int) * n);
  L->vnclass = (int *)malloc(sizeof(int) * n);
  L->skip = (int *)calloc(n, sizeof(int));
  if (!L->vclass || !L->vnclass || !L->skip) return 1;
  for (int r = 0; r < n; ++r) { L->vclass[r] = 3; L->vnclass[r] = l < C->nref ? 3 : 0; }
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        if (!(i == 0 || j == 0 || k == 0 || i == N - 1 || j == N - 1 || k == N - 1)) continue;
        int r = (k * N + j) * N + i;
        L->skip[r] = 1;
        for (int e = L->rowptr[r]; e < L->rowptr[r + 1]; ++e) L->val[e] = e == L->rowptr[r] ? 1.0 : 0.0;
      }
  /* standard transfer from level l-1 */
  L->prow = L->pcol = NULL;
  L->pw = NULL;
  if (l > 0) {
    const int Nc = (1 << (l - 1)) + 1;
    L->prow = (int *)malloc(sizeof(int) * (n + 1));
    L->pcol = (int *)malloc(sizeof(int) * (size_t)n * 2);
    L->pw = (double *)malloc(sizeof(double) * (size_t)n * 2);
    if (!L->prow || !L->pcol || !L->pw) return 1;
    int m = 0;
    L->prow[0] = 0;
    for (int k = 0; k < N; ++k)
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          int r = (k * N + j) * N + i, oi = i & 1, oj = j & 1, ok = k & 1;
          if (!oi && !oj && !ok) {
            L->pcol[m] = ((k / 2) * Nc + j / 2) * Nc + i / 2; L->pw[m++] = 1.0;
          } else {
            L->pcol[m] = (((k - ok) / 2) * Nc + (j - oj) / 2) * Nc + (i - oi) / 2; L->pw[m++] = 0.5;
            L->pcol[m] = (((k + ok) / 2) * Nc + (j + oj) / 2) * Nc + (i + oi) / 2; L->pw[m++] = 0.5;
          }
          L->prow[r + 1] = m;
        }
  }
  return 0;
}

/* ---- rule 1: UG's red refinement ----------------------------------------- */
static const int kEdge[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
/* sons of TET_RED_2_4, TET_RED_0_5, TET_RED_1_3: corners 0..3 of the father,
 * 4 + e the midpoint of edge e */
static const int kSons[3][8][4] = {
    {{0, 4, 6, 7}, {4, 5, 8, 1}, {5, 6, 9, 2}, {7, 8, 9, 3}, {4, 6, 7, 8}, {4, 5, 6, 8}, {5, 6, 8, 9}, {6, 7, 8, 9}},
    {{5, 6, 9, 2}, {4, 5, 8, 1}, {7, 8, 9, 3}, {0, 4, 6, 7}, {4, 5, 6, 9}, {5, 8, 9, 4}, {4, 7, 8, 9}, {4, 6, 7, 9}},
    {{7, 8, 9, 3}, {4, 5, 8, 1}, {0, 4, 6, 7}, {5, 6, 9, 2}, {5, 7, 8, 9}, {4, 5, 7, 8}, {4, 5, 6, 7}, {5, 6, 7, 9}}};
static int kOffs26[26][3];
static void init_offs26(void) {
  for (int q = 0; q < 14; ++q)
    for (int d = 0; d < 3; ++d) kOffs26[q][d] = kOffs[q][d];
  int q = 14;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        int nonneg = dx >= 0 && dy >= 0 && dz >= 0, nonpos = dx <= 0 && dy <= 0 && dz <= 0;
        if (nonneg || nonpos) continue; /* the origin and the 14 above */
        kOffs26[q][0] = dx; kOffs26[q][1] = dy; kOffs26[q][2] = dz; ++q;
      }
}
static int dir26(int dx, int dy, int dz) {
  for (int q = 0; q < 26; ++q)
    if (kOffs26[q][0] == dx && kOffs26[q][1] == dy && kOffs26[q][2] == dz) return q;
  return -1;
}

typedef struct { int c[4][3]; } tet;

/* index into kSons of the rule UG takes for a tetrahedron whose corners
 * and edge midpoints (in units of the son lattice) are P[0..9] */
static int shortest_interior_edge(int P[10][3]) {
  long long d[3] = {0, 0, 0}; /* squared lengths of the diagonals 0-5, 1-3, 2-4 */
  static const int ends[3][2] = {{4, 9}, {5, 7}, {6, 8}};
  for (int g = 0; g < 3; ++g)
    for (int x = 0; x < 3; ++x) {
      long long t = P[ends[g][0]][x] - P[ends[g][1]][x];
      d[g] += t * t;
    }
  int flags = (d[0] < d[1]) | ((d[1] < d[2]) << 1) | ((d[2] < d[0]) << 2);
  if (flags == 2 || flags == 6) return 2; /* TET_RED_1_3 */
  if (flags == 4 || flags == 5) return 0; /* TET_RED_2_4 */
  return 1;                               /* TET_RED_0_5 */
}

typedef struct { int z, y, x, ids[4]; int t; } elem_key;
static int cmp_int(const void *a, const void *b) { return *(const int *)a - *(const int *)b; }
static int cmp_key(const void *pa, const void *pb) {
  const elem_key *a = (const elem_key *)pa, *b = (const elem_key *)pb;
  if (a->z != b->z) return a->z < b->z ? -1 : 1;
  if (a->y != b->y) return a->y < b->y ? -1 : 1;
  if (a->x != b->x) return a->x < b->x ? -1 : 1;
  for (int i = 0; i < 4; ++i)
    if (a->ids[i] != b->ids[i]) return a->ids[i] < b->ids[i] ? -1 : 1;
  return 0;
}

typedef struct { const field *F; double h; const tet *T; const elem_key *K; size_t e0, e1; double *kc; } ug_field_job;
static void *ug_field_range(void *arg) {
  ug_field_job *J = (ug_field_job *)arg;
  for (size_t e = J->e0; e < J->e1; ++e) {
    const tet *t = &J->T[J->K[e].t];
    double xc[3] = {0, 0, 0};
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) xc[d] += (t->c[a][d] * J->h) / 4;
    J->kc[e] = field_k(J->F, xc);
  }
  return NULL;
}

/* level l of rule 1 from its tetrahedra; nb[] receives the 26-bit
 * neighbour masks, cnb[] holds level l-1's */
static int build_level_ug(orc_cube *C, int l, const tet *T, size_t nt_el, const uint32_t *cnb, uint32_t *nb,
                          const field *F, int nthreads) {
  level *L = &C->lev[l];
  const int N = (1 << l) + 1, n = N * N * N, nc = N - 1;
  const double h = 1.0 / (N - 1);
  L->N = N;
  L->n = n;
  memset(nb, 0, sizeof(uint32_t) * (size_t)n);
  for (size_t e = 0; e < nt_el; ++e)
    for (int g = 0; g < 6; ++g) {
      const int *a = T[e].c[kEdge[g][0]], *b = T[e].c[kEdge[g][1]];
      int fwd = dir26(b[0] - a[0], b[1] - a[1], b[2] - a[2]), bwd = dir26(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
      if (fwd < 0 || bwd < 0) return 1; /* an edge longer than one lattice step */
      nb[(a[2] * N + a[1]) * N + a[0]] |= 1u << fwd;
      nb[(b[2] * N + b[1]) * N + b[0]] |= 1u << bwd;
    }
  size_t nnz = 0;
  for (int r = 0; r < n; ++r) nnz += 1 + (size_t)__builtin_popcount(nb[r]);
  L->rowptr = (int *)malloc(sizeof(int) * (n + 1));
  L->col = (int *)malloc(sizeof(int) * nnz);
  L->xyz = (double *)malloc(sizeof(double) * (size_t)n * 3);
  int *pos = (int *)malloc(sizeof(int) * (size_t)n * 26);
  if (!L->rowptr || !L->col || !L->xyz || !pos) { free(pos); return 1; }
  int q = 0;
  L->rowptr[0] = 0;
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        int r = (k * N + j) * N + i;
        L->xyz[(size_t)r * 3] = i * h; L->xyz[(size_t)r * 3 + 1] = j * h; L->xyz[(size_t)r * 3 + 2] = k * h;
        L->col[q++] = r;
        for (int o = 0; o < 26; ++o) {
          pos[(size_t)r * 26 + o] = -1;
          if (!(nb[r] >> o & 1u)) continue;
          pos[(size_t)r * 26 + o] = q;
          L->col[q++] = ((k + kOffs26[o][2]) * N + j + kOffs26[o][1]) * N + i + kOffs26[o][0];
        }
        L->rowptr[r + 1] = q;
      }
  /* elements in summation order */
  elem_key *K = (elem_key *)malloc(sizeof(elem_key) * (nt_el ? nt_el : 1));
  double *kc = (double *)malloc(sizeof(double) * (nt_el ? nt_el : 1));
  L->val = (double *)calloc((size_t)q, sizeof(double));
  if (!K || !kc || !L->val) { free(K); free(kc); free(pos); return 1; }
  for (size_t e = 0; e < nt_el; ++e) {
    elem_key *k = &K[e];
    k->x = k->y = k->z = 1 << 30;
    for (int a = 0; a < 4; ++a) {
      const int *v = T[e].c[a];
      if (v[0] < k->x) k->x = v[0];
      if (v[1] < k->y) k->y = v[1];
      if (v[2] < k->z) k->z = v[2];
      k->ids[a] = (v[2] * N + v[1]) * N + v[0];
    }
    qsort(k->ids, 4, sizeof(int), cmp_int);
    k->t = (int)e;
  }
  qsort(K, nt_el, sizeof(elem_key), cmp_key);
  int nt = nthreads < 1 ? 1 : nthreads > 64 ? 64 : nthreads;
  pthread_t th[64];
  ug_field_job jobs[64];
  for (int w = 0; w < nt; ++w) {
    jobs[w].F = F; jobs[w].h = h; jobs[w].T = T; jobs[w].K = K; jobs[w].kc = kc;
    jobs[w].e0 = nt_el * w / nt; jobs[w].e1 = nt_el * (w + 1) / nt;
  }
  for (int w = 1; w < nt; ++w) pthread_create(&th[w], NULL, ug_field_range, &jobs[w]);
  ug_field_range(&jobs[0]);
  for (int w = 1; w < nt; ++w) pthread_join(th[w], NULL);
  for (int parity = 0; parity < 2; ++parity)
    for (size_t e = 0; e < nt_el; ++e) {
      if ((K[e].z & 1) != parity) continue;
      const tet *t = &T[K[e].t];
      double X[4][3], Ke[16];
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) X[a][d] = t->c[a][d] * h;
      p1_stiffness(X, kc[e], Ke);
      for (int a = 0; a < 4; ++a) {
        const int *va = t->c[a];
        int r = (va[2] * N + va[1]) * N + va[0];
        for (int b = 0; b < 4; ++b) {
          const int *vb = t->c[b];
          int ent = a == b ? L->rowptr[r] : pos[(size_t)r * 26 + dir26(vb[0] - va[0], vb[1] - va[1], vb[2] - va[2])];
          L->val[ent] += Ke[a * 4 + b];
        }
      }
    }
  free(K);
  free(kc);
  free(pos);
  L->vclass = (int *)malloc(sizeof(int) * n);
  L->vnclass = (int *)malloc(sizeof(int) * n);
  L->skip = (int *)calloc(n, sizeof(int));
  if (!L->vclass || !L->vnclass || !L->skip) return 1;
  for (int r = 0; r < n; ++r) { L->vclass[r] = 3; L->vnclass[r] = l < C->nref ? 3 : 0; }
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        if (!(i == 0 || j == 0 || k == 0 || i == N - 1 || j == N - 1 || k == N - 1)) continue;
        int r = (k * N + j) * N + i;
        L->skip[r] = 1;
        for (int e = L->rowptr[r]; e < L->rowptr[r + 1]; ++e) L->val[e] = e == L->rowptr[r] ? 1.0 : 0.0;
      }
  L->prow = L->pcol = NULL;
  L->pw = NULL;
  if (l == 0) return 0;
  const int Nc = (1 << (l - 1)) + 1;
  L->prow = (int *)malloc(sizeof(int) * (n + 1));
  L->pcol = (int *)malloc(sizeof(int) * (size_t)n * 2);
  L->pw = (double *)malloc(sizeof(double) * (size_t)n * 2);
  if (!L->prow || !L->pcol || !L->pw) return 1;
  int m = 0;
  L->prow[0] = 0;
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        int r = (k * N + j) * N + i, p[3] = {i, j, k};
        if (!(i & 1) && !(j & 1) && !(k & 1)) {
          L->pcol[m] = ((k / 2) * Nc + j / 2) * Nc + i / 2; L->pw[m++] = 1.0;
          L->prow[r + 1] = m;
          continue;
        }
        /* the coarse edges through p: for each odd axis, the end a steps
         * down (sign bit 0) or up (bit 1) and the end b the other way */
        int found = 0;
        for (int sg = 0; sg < 8 && !found; ++sg) {
          int a[3], b[3], ok = 1;
          for (int d = 0; d < 3; ++d) {
            if (!(p[d] & 1)) { if (sg >> d & 1) ok = 0; a[d] = b[d] = p[d] / 2; continue; }
            int s = (sg >> d & 1) ? -1 : 1;
            a[d] = (p[d] - s) / 2;
            b[d] = (p[d] + s) / 2;
          }
          if (!ok) continue;
          int o = dir26(b[0] - a[0], b[1] - a[1], b[2] - a[2]);
          if (o < 0 || !(cnb[(a[2] * Nc + a[1]) * Nc + a[0]] >> o & 1u)) continue;
          L->pcol[m] = (a[2] * Nc + a[1]) * Nc + a[0]; L->pw[m++] = 0.5;
          L->pcol[m] = (b[2] * Nc + b[1]) * Nc + b[0]; L->pw[m++] = 0.5;
          found = 1;
        }
        if (!found) return 1;
        L->prow[r + 1] = m;
      }
  return 0;
}

static int build_ug(orc_cube *C, const field *F, int nthreads) {
  static const int cube[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  static const int coarse[6][4] = {{0, 1, 2, 6}, {0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 4, 5, 6}, {0, 5, 1, 6}};
  init_offs26();
  size_t ne = 6, nmax = (size_t)6 << (3 * C->nref);
  const size_t nn = (size_t)((1 << C->nref) + 1) * ((1 << C->nref) + 1) * ((1 << C->nref) + 1);
  tet *T = (tet *)malloc(sizeof(tet) * nmax), *S = (tet *)malloc(sizeof(tet) * nmax);
  uint32_t *nb = (uint32_t *)malloc(sizeof(uint32_t) * nn), *cnb = (uint32_t *)malloc(sizeof(uint32_t) * nn);
  int rc = !T || !S || !nb || !cnb;
  if (!rc) {
    for (int e = 0; e < 6; ++e)
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) T[e].c[a][d] = cube[coarse[e][a]][d];
    rc = build_level_ug(C, 0, T, ne, NULL, nb, F, nthreads);
  }
  for (int l = 1; l <= C->nref && !rc; ++l) {
    for (size_t e = 0; e < ne; ++e) {
      int P[10][3];
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) P[a][d] = 2 * T[e].c[a][d];
      for (int g = 0; g < 6; ++g)
        for (int d = 0; d < 3; ++d) P[4 + g][d] = T[e].c[kEdge[g][0]][d] + T[e].c[kEdge[g][1]][d];
      const int r = shortest_interior_edge(P);
      for (int s = 0; s < 8; ++s)
        for (int a = 0; a < 4; ++a)
          for (int d = 0; d < 3; ++d) S[e * 8 + s].c[a][d] = P[kSons[r][s][a]][d];
    }
    ne *= 8;
    tet *x = T; T = S; S = x;
    uint32_t *y = cnb; cnb = nb; nb = y;
    rc = build_level_ug(C, l, T, ne, cnb, nb, F, nthreads);
  }
  free(T); free(S); free(nb); free(cnb);
  return rc;
}

int orc_cube_create(int nref, unsigned long long seed, double corr, double var, int nthreads, orc_cube **out) {
  return orc_cube_create_rule(0, nref, seed, corr, var, nthreads, out);
}

int orc_cube_create_rule(int rule, int nref, unsigned long long seed, double corr, double var, int nthreads,
                         orc_cube **out) {
  if (!out || rule < 0 || rule > 1 || nref < 0 || nref > (rule ? 7 : 8)) return 1;
  init_offs();
  orc_cube *C = (orc_cube *)calloc(1, sizeof *C);
  if (!C) return 1;
  C->nref = nref;
  C->lev = (level *)calloc(nref + 1, sizeof(level));
  field *F = (field *)malloc(sizeof(field));
  if (!C->lev || !F) { free(F); orc_cube_destroy(C); return 1; }
  field_init(F, seed, corr, var);
  if (rule == 1) {
    if (build_ug(C, F, nthreads)) { free(F); orc_cube_destroy(C); return 1; }
  } else {
    for (int l = 0; l <= nref; ++l)
      if (build_level(C, l, F, nthreads)) { free(F); orc_cube_destroy(C); return 1; }
  }
  free(F);
  const level *T = &C->lev[nref];
  const double scale = (double)(1 << nref), hd = pow(1.0 / scale, 3);
  C->rhs_len = T->n;
  C->rhs = (double *)malloc(sizeof(double) * T->n);
  if (!C->rhs) { orc_cube_destroy(C); return 1; }
  for (int r = 0; r < T->n; ++r) {
    int i = r % T->N, j = (r / T->N) % T->N, k = r / (T->N * T->N);
    C->rhs[r] = T->skip[r] ? 0.0 : rhs_uniform(seed, lattice_key(i, j, k)) * hd;
  }
  *out = C;
  return 0;
}

int orc_cube_level(const orc_cube *C, int l, orc_level *out, const double **xyz) {
  if (!C || l < 0 || l > C->nref || !out) return 1;
  const level *L = &C->lev[l];
  out->n = L->n; out->s = 1;
  out->rowptr = L->rowptr; out->col = L->col; out->val = L->val;
  out->vclass = L->vclass; out->vnclass = L->vnclass; out->skip = L->skip;
  out->prowptr = L->prow; out->pcol = L->pcol; out->pw = L->pw;
  if (xyz) *xyz = L->xyz;
  return 0;
}

const double *orc_cube_rhs(const orc_cube *C, int *len) {
  if (!C) return NULL;
  if (len) *len = C->rhs_len;
  return C->rhs;
}

void orc_cube_destroy(orc_cube *C) {
  if (!C) return;
  if (C->lev)
    for (int l = 0; l <= C->nref; ++l) {
      level *L = &C->lev[l];
      free(L->rowptr); free(L->col); free(L->val); free(L->vclass); free(L->vnclass); free(L->skip);
      free(L->prow); free(L->pcol); free(L->pw); free(L->xyz);
    }
  free(C->lev);
  free(C->rhs);
  free(C);
}
