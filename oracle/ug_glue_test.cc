// ug_glue_test: drives UG 3.12.1 (built from its sources by oracle/Makefile)
// with the GB300 numproc classes of ug_gb300/ug_glue/gpu_numprocs.cc.
// TEST INFRASTRUCTURE: checks, on a host without a GPU, that the glue
// compiles against UG's headers and links with libug_gb300, that UG's own
// script commands resolve to its classes, that its flattening walks UG's
// lists, and that the library's errors come back through UG's numproc
// error path.  Prints one line per check; exit code 0 = every check held.
//
// The problem: the unit square, one Q1 quadrilateral refined 4 times, the
// Q1 Laplacian assembled on every level with homogeneous Dirichlet rows.
#include <config.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "cmdint.h"
#include "commands.h"
#include "gm.h"
#include "initug.h"
#include "iter.h"
#include "ls.h"
#include "np.h"
#include "numproc.h"
#include "std_domain.h"
#include "udm.h"
#include "ugdevices.h"

USING_UG_NAMESPACES

INT InitGpuNumProcs(void);
INT GpuNumProcsFlatten(MULTIGRID *mg, MATDATA_DESC *A, INT level, INT *nlevels, INT *n, INT *nnz, INT *npw);

static INT BndCond(void *, void *, DOUBLE *, DOUBLE *value, INT *type) { value[0] = 0.0; type[0] = 0; return 0; }

static int g_fail = 0;
static void check(bool ok, const char *what) {
  printf("%s %s\n", ok ? "ok" : "FAIL", what);
  if (!ok) g_fail = 1;
}
static INT cmd(const char *c) {
  char b[1024];
  snprintf(b, sizeof b, "%s", c);
  return InterpretCommand(b);
}

int main(int argc, char **argv) {
  INT ac = 1;
  char *a0 = argv[0];
  char **av = &a0;
  if (InitUg(&ac, &av)) { printf("FAIL InitUg\n"); return 1; }
  check(InitGpuNumProcs() == 0, "InitGpuNumProcs registers the classes");

  CreateBoundaryValueProblem("bvp", BndCond, 0, NULL, 0, NULL);
  const char *setup[] = {"configure bvp $d Quadrilateral;", "newformat fmt $V n1: vt 20 $M implicit(vt): mt 4;",
                         "new mg $b bvp $f fmt $h 500M;", "ie 0 1 2 3;", "fixcoarsegrid;"};
  for (const char *c : setup)
    if (cmd(c)) { printf("FAIL %s\n", c); return 1; }
  for (int l = 0; l < 4; ++l)
    if (cmd("mark $a;") || cmd("refine;")) { printf("FAIL refine\n"); return 1; }
  if (cmd("createvector sol rhs; creatematrix MAT;")) { printf("FAIL createvector\n"); return 1; }
  MULTIGRID *mg = GetCurrentMultigrid();
  MATDATA_DESC *A = GetMatDataDescByName(mg, (char *)"MAT");
  const SHORT *mc = MD_MCMPPTR_OF_RT_CT(A, NODEVEC, NODEVEC);
  static const double K[4][4] = {{4, -1, -2, -1}, {-1, 4, -1, -2}, {-2, -1, 4, -1}, {-1, -2, -1, 4}};
  for (int l = 0; l <= TOPLEVEL(mg); ++l) {
    GRID *g = GRID_ON_LEVEL(mg, l);
    for (VECTOR *v = FIRSTVECTOR(g); v; v = SUCCVC(v)) {
      VECSKIP(v) = 0;
      for (MATRIX *m = VSTART(v); m; m = MNEXT(m)) MVALUE(m, mc[0]) = 0.0;
    }
    for (ELEMENT *e = FIRSTELEMENT(g); e; e = SUCCE(e)) {
      VECTOR *vv[4];
      for (int i = 0; i < 4; ++i) vv[i] = NVECTOR(CORNER(e, i));
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) MVALUE(i == j ? VSTART(vv[i]) : GetMatrix(vv[i], vv[j]), mc[0]) += K[i][j] / 6.0;
    }
    for (NODE *n = FIRSTNODE(g); n; n = SUCCN(n))
      if (OBJT(MYVERTEX(n)) == BVOBJ) {
        VECTOR *v = NVECTOR(n);
        VECSKIP(v) = 1;
        MVALUE(VSTART(v), mc[0]) = 1.0;
        for (MATRIX *m = MNEXT(VSTART(v)); m; m = MNEXT(m)) MVALUE(m, mc[0]) = 0.0;
      }
  }

  // the flattening the device would receive: UG's level sizes and patterns
  INT nl = 0, n = 0, nnz = 0, npw = 0;
  check(GpuNumProcsFlatten(mg, A, 4, &nl, &n, &nnz, &npw) == 0 && nl == 5 && n == 289 && nnz == 2401,
        "flattening: 5 levels, 17x17 top level with the Q1 pattern (9-point rows)");
  // 289 top-level vectors: 81 corner copies (one weight), 144 edge midpoints (two), 64 cell centres (four)
  check(npw == 81 + 2 * 144 + 4 * 64, "flattening: standard transfer weights of the top level");

  // UG's script with the GB300 class names
  const char *script[] = {
      "npcreate transfer $c gtransfer;", "npinit transfer;", "npcreate smooth $c gjac;", "npinit smooth $damp 0.8;",
      "npcreate base $c gex;", "npinit base;", "npcreate basesolver $c gls;",
      "npinit basesolver $red 1e-14 $m 1 $I base;", "npcreate lmgc $c glmgc;",
      "npinit lmgc $S smooth smooth basesolver $T transfer $n1 2 $n2 2 $b 1;", "npcreate mgs $c gls;",
      "npinit mgs $A MAT $x sol $b rhs $red 1e-10 $m 50 $I lmgc;"};
  bool all = true;
  for (const char *c : script) all = all && cmd(c) == 0;
  check(all, "npcreate / npinit of gtransfer, gjac, gex, gls, glmgc");
  NP_BASE *ls = GetNumProcByName(mg, "mgs", LINEAR_SOLVER_CLASS_NAME);
  check(ls && strcmp(ENVITEM_NAME(ls), "linear_solver.gls.mgs") == 0 && ls->status == NP_EXECUTABLE,
        "mgs is a linear_solver.gls object, EXECUTABLE");
  NP_BASE *it = GetNumProcByName(mg, "lmgc", ITER_CLASS_NAME);
  check(it && strcmp(ENVITEM_NAME(it), "iter.glmgc.lmgc") == 0 && ((NP_ITER *)it)->Iter != NULL,
        "lmgc is an iter.glmgc object with its Iter forwarder");
  check(cmd("npdisplay mgs;") == 0, "npdisplay of a GB300 object");

  // a solve without a CUDA device: the library's failure returns through
  // NP_RETURN and UG's command fails (it must not abort)
  check(cmd("npexecute mgs $i $d $r $s $p;") != 0, "npexecute without a device: UG reports the numproc error");
  return g_fail;
}
