/* lmgc_oracle: a plain-C, sequential restatement of UG 3.12.1's linear
 * multigrid path (ls + lmgc with jac / gs / ilu smoothers, the standard
 * transfer and the ex base solver) on a flattened hierarchy.
 *
 * TEST INFRASTRUCTURE ONLY.  It is the oracle the CUDA path is compared
 * against (tests/, __graft_entry__.smoke, and bench.py's CPU baseline leg);
 * the ug_gb300 product never calls it.  Its own correctness is pinned
 * against golden vectors produced by the UG reference itself
 * (oracle/ug_export.cc -> tests/golden/).
 *
 * Layout: one level = block CSR in UG's VECTOR-list order, each row's
 * MATRIX list in VSTART/MNEXT order (diagonal block first), blocks stored
 * row-major (s*s doubles), plus the VCLASS / VNCLASS / VECSKIP fields and
 * the standard-transfer weights to the next coarser level as a CSR over the
 * fine vectors.  Every function is re-entrant (no global state), so
 * independent solves may run concurrently on different threads. */
#ifndef LMGC_ORACLE_H
#define LMGC_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_S 8

typedef struct {
  int n;              /* block rows (VECTORs) */
  int s;              /* block size (components per VECTOR) */
  const int *rowptr;  /* n+1 */
  const int *col;     /* nnzb, diagonal first in each row */
  const double *val;  /* nnzb*s*s */
  const int *vclass;  /* VCLASS per vector (ACTIVE_CLASS = 3, NEWDEF_CLASS = 2) */
  const int *vnclass; /* VNCLASS per vector */
  const int *skip;    /* VECSKIP bit mask per vector */
  /* standard transfer from level-1 to this level; NULL on the coarsest */
  const int *prowptr; /* n+1 */
  const int *pcol;    /* coarse vector index */
  const double *pw;   /* weight (1 for a corner copy, else shape function) */
} orc_level;

enum { ORC_JAC = 0, ORC_GS = 1, ORC_ILU = 2 };

/* An interpolation matrix of a fine level (UG's IMATRIX: the VISTART list of
 * every fine VECTOR): per fine vector (CSR over the fine level, list order)
 * the coarse vectors it couples to, each with an s x s block stored coarse
 * component major (val[k*s*s + i*s + j]: coarse component i, fine
 * component j), as MVALUE of an interpolation matrix. */
typedef struct {
  const int *rowptr;  /* fine n + 1 */
  const int *col;     /* coarse vector index */
  const double *val;  /* rowptr[n] * s * s */
} orc_imat;

typedef struct {
  int nlevels;            /* levels 0..nlevels-1 */
  const orc_level *lev;
  int baselevel;          /* lmgc $b */
  int nu1, nu2, gamma;    /* lmgc $n1 $n2 $g */
  int smoother;           /* ORC_JAC / ORC_GS / ORC_ILU, same for pre and post */
  double damp[ORC_MAX_S]; /* smoother $damp */
  double beta[ORC_MAX_S]; /* ilu $beta */
  double cdamp[ORC_MAX_S];/* lmgc $damp (interpolation damping) */
  /* the base solver is an `ls` ($m 1, $I ex): it does nothing when every
   * component of the base-level defect is already below its abslimit
   * (default ABS_LIMIT = 1e-10, np/procs/ls.cc:66, 389-391, 689) */
  double base_abslimit[ORC_MAX_S];
  /* the transfer's matrix mode (`npinit transfer $M`): imat[l] is level l's
   * interpolation matrix (l >= 1), used for RestrictDefect and
   * InterpolateCorrection instead of the standard weights; NULL = standard */
  const orc_imat *imat;
} orc_mg;

/* ---- kernels (one level) ---- */
void orc_matmul_minus(const orc_level *L, double *x, const double *y);          /* x -= A y */
int orc_jac(const orc_level *L, double *v, const double *d);                      /* l_jac */
int orc_lgs(const orc_level *L, double *v, const double *d);                      /* l_lgs */
int orc_ilu_decomp(const orc_level *L, double *lu, const double *beta);           /* l_ilubthdecomp */
int orc_luiter(const orc_level *L, const double *lu, double *v, const double *d); /* l_luiter */
void orc_nrm2x(const orc_level *L, const double *x, double *out);                 /* dnrm2x */
void orc_restrict(const orc_level *fine, const orc_level *coarse, double *to_coarse,
                  const double *from_fine, const double *damp);                   /* StandardRestrict */
void orc_interpolate(const orc_level *fine, double *to_fine, const double *from_coarse,
                     const double *damp);                                         /* StandardInterpolateCorrection */
void orc_interpolate_new(const orc_level *fine, const int *vnew, double *x_fine,
                         const double *x_coarse);                                 /* StandardIntNewNodeVector */
void orc_project(const orc_level *fine, double *x_coarse, const double *x_fine);  /* StandardProject */
void orc_restrict_imat(const orc_level *fine, const orc_imat *M, const orc_level *coarse, double *to_coarse,
                       const double *from_fine, const double *damp);              /* RestrictByMatrix */
void orc_interpolate_imat(const orc_level *fine, const orc_imat *M, double *to_fine, const double *from_coarse,
                          const double *damp);
/* InterpolateNewVectorsByMatrix (transgrid.cc:1425): the VNEW fine vectors
 * from the coarse level through the interpolation matrix */
void orc_interpolate_new_imat(const orc_level *fine, const orc_imat *M, const int *vnew, double *x_fine,
                              const double *x_coarse);                                    /* InterpolateCorrectionByMatrix */

/* ---- solver ----
 * Solves A x = b on level top = nlevels-1 with ls + lmgc.  x (finest, n*s)
 * is the start value and receives the solution; b is overwritten by the
 * final defect.  hist (may be NULL) receives s*(maxit+1) defect norms.
 * Returns the number of iterations, or a negative error code. */
/* The same problem with UG's cg (np/procs/ls.cc:901-1064, CGPrepare /
 * CGUpdate in LinearSolver's loop) preconditioned by lmgc. */
int orc_cg_solve(const orc_mg *mg, double *x, double *b, const double *red, const double *abslimit, int maxit,
                 double *hist, int *converged);
/* ... and with UG's bcgs (ls.cc:1711-2062, BiCGStab with the lmgc preconditioner,
 * two half steps per iteration, each counted; hist holds one entry per half step). */
int orc_bcgs_solve(const orc_mg *mg, double *x, double *b, const double *red, const double *abslimit, int maxit,
                   double *hist, int *converged);
int orc_ls_solve(const orc_mg *mg, double *x, double *b, const double *red, const double *abslimit,
                 int maxit, double *hist, int *converged);
/* ls + lmgc on a locally refined hierarchy: x[l] and b[l] for every level
 * l = 0..top.  The defect and its norm run over UG's surface (ON_SURFACE:
 * FINE_GRID_DOF vectors of the levels FULLREFINELEVEL..top-1 and NEW_DEFECT
 * vectors of the top level, each row with its own level's matrix), and
 * LSUpdate adds the correction on every level baselevel..top (ls.cc:562,
 * 577, 869).  On a uniformly refined hierarchy it equals orc_ls_solve. */
int orc_ls_solve_levels(const orc_mg *mg, double *const *x, double *const *b, const double *red,
                        const double *abslimit, int maxit, double *hist, int *converged);
int orc_fullrefinelevel(const orc_mg *mg); /* SetSurfaceClasses, gm/algebra.cc:2838 */
/* cg and bcgs (ls.cc:989-1030, 1864-2062) on every level baselevel..top:
 * vector operations ALL_VECTORS on each level, dot products (ddot / ddotw)
 * and bcgs's dmatmul ON_SURFACE, as UG runs them on a locally refined grid. */
int orc_cg_solve_levels(const orc_mg *mg, double *const *x, double *const *b, const double *red,
                        const double *abslimit, int maxit, double *hist, int *converged);
int orc_bcgs_solve_levels(const orc_mg *mg, double *const *x, double *const *b, const double *red,
                          const double *abslimit, int maxit, double *hist, int *converged);

#ifdef __cplusplus
}
#endif
#endif
