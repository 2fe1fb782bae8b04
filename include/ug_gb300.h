/*
 * ug_gb300.h -- C ABI of the GB300 (sm_103a) implementation of UG's linear
 * multigrid hot path: lmgc with the jac / gs / ilu smoothers, the standard
 * grid transfer, the ex base solver and the ls outer iteration.
 *
 * The boundary mirrors UG 3.12.1's numproc plugin interface
 * (np/udm/numproc.h, np/procs/iter.h, transfer.h, ls.h): a UG build adds
 * numproc classes whose function pointers forward to the gmg_iter_* /
 * gmg_transfer_* / gmg_ls_* entry points below, after flattening its
 * VECTOR/MATRIX lists into gmg_level_desc arrays at every grid change.
 *
 * Conventions (those of the reference):
 *   - every entry point returns 0 on success and nonzero on failure, never
 *     aborts; gmg_last_error() describes the last failure of this thread;
 *   - `result` out-parameters receive an error code as NP_RETURN does
 *     (np/np.h:89); a failed decomposition reports -(row index+1);
 *   - levels are numbered 0 (coarsest) .. nlevels-1 (finest);
 *   - host arrays are in UG's VECTOR-list order; each MATRIX row lists the
 *     diagonal block first (VSTART), then the off-diagonal blocks (MNEXT);
 *     blocks are row-major s*s; vectors hold s components per VECTOR.
 * All pointers are plain host pointers unless the name says _dev.
 */
#ifndef UG_GB300_H
#define UG_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define GMG_MAX_S 8   /* largest block size (components per VECTOR) */

typedef struct gmg_mg gmg_mg;   /* multigrid: device hierarchy + user data + numprocs (MULTIGRID) */
typedef struct gmg_vec gmg_vec; /* vector data descriptor, one array per level (VECDATA_DESC) */
typedef struct gmg_mat gmg_mat; /* matrix data descriptor (MATDATA_DESC) */
typedef struct gmg_np gmg_np;   /* numproc object (NP_BASE and derived) */

/* LRESULT, np/procs/ls.h:71-77 */
typedef struct {
  int error_code;
  int converged;
  double first_defect[GMG_MAX_S];
  double last_defect[GMG_MAX_S];
  int number_of_linear_iterations;
} gmg_lresult;

/* One level of the flattened hierarchy (host arrays, UG VECTOR-list order).
 * Produced from VSTART/MNEXT/MDEST/MVALUE (gm/gm.h:601-672), VCLASS/VNCLASS
 * (gm.h:2200-2207), VECSKIP (gm.h:2286) and the standard transfer weights
 * (corner node -> father copy with weight 1, other nodes -> father element
 * corners with the shape functions GNs at LCVECT, np/algebra/transgrid.cc:117). */
typedef struct {
  int n;               /* VECTORs on the level */
  int s;               /* components per VECTOR (block size), 1..GMG_MAX_S */
  const int *rowptr;   /* n+1 */
  const int *col;      /* rowptr[n] block column indices, diagonal first in each row */
  const double *val;   /* rowptr[n]*s*s values */
  const int *vclass;   /* n, or NULL for all 3 (ACTIVE_CLASS) */
  const int *vnclass;  /* n, or NULL for all 3 */
  const int *skip;     /* n VECSKIP masks, or NULL for none */
  const int *prowptr;  /* standard transfer from level-1: n+1 (NULL on level 0) */
  const int *pcol;     /* coarse VECTOR index per weight */
  const double *pw;    /* weight */
} gmg_level_desc;

/* processing order of every level (the `order` numproc, np/procs/order.cc) */
#define GMG_ORDER_LIST 0  /* UG's VECTOR-list order: gs / ilu reproduce l_lgs / l_luiter */
#define GMG_ORDER_COLOR 1 /* multicolour order (greedy colouring of the matrix graph) */
#define GMG_ORDER_DOMAIN 2 /* subdomain order: interiors of small breadth-first subdomains, then the
                              coloured interface rows (level-scheduled ILU / GS with few wavefronts) */

#define GMG_PREC_FP64 0
#define GMG_PREC_FP32 1

typedef struct {
  int order;        /* GMG_ORDER_* */
  int fp32_copy;    /* also keep FP32 copies of matrices/transfers (mixed precision) */
  int autotune;     /* time each level's kernel variants at creation and keep the fastest */
  int device;       /* CUDA device ordinal */
  int disable_pdl;  /* 1: launch without programmatic dependent launch */
} gmg_mg_opts;

/* ---------------------------------------------------------------- setup */
/* Flattened hierarchy -> device (a grid change: AdaptMultiGrid, gm/refine.cc:6482,
 * followed by assembly).  Creates the system matrix descriptor "MAT". */
int gmg_mg_create(const gmg_level_desc *levels, int nlevels, const gmg_mg_opts *opts, gmg_mg **out);
int gmg_mg_destroy(gmg_mg *mg);
/* Runs all of mg's work on this CUDA stream (cudaStream_t; NULL = legacy default). */
int gmg_mg_set_stream(gmg_mg *mg, void *stream);
int gmg_mg_nlevels(const gmg_mg *mg);
int gmg_mg_level_size(const gmg_mg *mg, int level, int *n, int *s, long long *nnzb);
/* perm[i] = UG list position of the VECTOR processed i-th on this level */
int gmg_mg_get_order(const gmg_mg *mg, int level, int *perm);
/* The matrix as stored on the device, in processing order (for checking). */
int gmg_mg_get_matrix(const gmg_mg *mg, int level, int *rowptr, int *col, double *val);
/* Number of multicolour classes (wavefronts of the gs/ilu schedule) on a level. */
int gmg_mg_num_waves(const gmg_mg *mg, int level);
/* Host vectors (uploads, downloads, gmg_solve_host): 1 = copied straight
 * from / to the caller's pageable memory, the default where the device reads
 * host memory through the host's page tables (Grace); 0 = through a pinned
 * staging buffer, the default elsewhere.  Same results. */
int gmg_mg_set_direct_host(gmg_mg *mg, int on);
/* Interface sweeps of the subdomain order (ILU in GMG_ORDER_DOMAIN): all
 * interface colours of a direction in one cooperative launch, rows waiting
 * on their earlier-colour neighbours' completion flags, or one launch per
 * colour.  mode 0: per colour; 1 (default): one launch for FP64 sweeps, per
 * colour for FP32 ones (faster there); 2: one launch for both.
 * Bit-identical; set before the first graph-captured solve. */
int gmg_mg_set_iface_sweep(gmg_mg *mg, int mode);
/* The colouring GMG_ORDER_COLOR uses, on the host (no device needed):
 * DSATUR on the symmetrised graph of the CSR pattern (rowptr[n+1], col),
 * then a bounded, deterministic tabu search removing colours while it can.
 * colour[i] in 0..*ncolours-1; adjacent rows never share a colour. */
int gmg_colour_graph(int n, const int *rowptr, const int *col, int *colour, int *ncolours);
/* Subdomain order (GMG_ORDER_DOMAIN) of a level: subdomains, interior rows
 * and interface colours (all 0 in the other orders). */
int gmg_mg_domain_info(const gmg_mg *mg, int level, int *nsub, int *ninterior, int *ncolours);
/* The kernel variant a level runs: threads per row (CSR levels, 0 on
 * sliced-ELLPACK levels), row structure prefetched before the launch wait and
 * evict-first matrix stream (1 / 0, -1 = chosen by size); set by the
 * autotuner (gmg_mg_opts.autotune) at creation. */
int gmg_mg_level_variant(const gmg_mg *mg, int level, int *tpr, int *prefetch, int *stream);
/* How the chained Gauss-Seidel steps of a multicolour level (at most 48
 * colours) run: 0 = one launch per colour wave; 1 = ONE thread block, the
 * colour waves separated by block barriers (t and c within 200 KB of shared
 * memory); 2, 4, 8 or 16 = one thread-block cluster of that many blocks,
 * each holding all of t in shared memory (within 227 KB with its rows' c),
 * the waves separated by cluster barriers, new values sent to every block
 * through distributed shared memory.  All forms are bit-identical to the
 * per-wave launches.  The autotuner picks the fastest; set it before the
 * first solve that captures a CUDA graph.  Refused (1) for a level or device
 * where the form cannot run. */
int gmg_mg_level_cta_chain(const gmg_mg *mg, int level, int *on);
int gmg_mg_set_level_cta_chain(gmg_mg *mg, int level, int on);
/* Device bytes held by the hierarchy. */
long long gmg_mg_device_bytes(const gmg_mg *mg);
/* Kernel launches issued by mg since creation (or the last reset). */
long long gmg_mg_launch_count(const gmg_mg *mg, int reset);
const char *gmg_last_error(void);
/* Synchronise mg's stream; returns nonzero if a kernel failed or a bounded
 * device-side wait (the one-launch interface ILU sweeps) gave up. */
int gmg_mg_sync(gmg_mg *mg);

/* ------------------------------------------------ batched hierarchies */
/* `ninst` independent problems, instance k given as inst_nlevels[k] levels
 * (instances[k][0..]), all with one block size, stored block-diagonally:
 * level l of the result is the concatenation, in instance order, of level l
 * of every instance that has one, so each instance advances through the
 * same per-level kernels at once (no UG counterpart: UG solves one
 * MULTIGRID at a time; each instance is what UG's ls would compute for it).
 * Instance k's finest level inst_nlevels[k]-1 is its surface: every row there
 * has VNCLASS < 2 (UG's top level) and every row below has VNCLASS >= 2
 * (NULL vnclass arrays mean exactly that).  An ls on such a hierarchy, run
 * at its deepest level, tests convergence per instance and leaves converged
 * instances' x alone; vectors are passed packed (below). */
int gmg_mg_create_batched(const gmg_level_desc *const *instances, const int *inst_nlevels, int ninst,
                          const gmg_mg_opts *opts, gmg_mg **out);
/* number of instances (0 for a hierarchy from gmg_mg_create) */
int gmg_mg_num_instances(const gmg_mg *mg);
/* instance k's finest level, its VECTORs there and its first VECTOR in the packed layout */
int gmg_mg_instance_info(const gmg_mg *mg, int k, int *top, int *n_top, long long *pack_offset);
/* packed vectors: every instance's finest-level values (its list order, s per
 * VECTOR), instance after instance: sum_k n_top[k]*s doubles; synchronous */
int gmg_vec_upload_packed(gmg_vec *v, const double *host);
int gmg_vec_download_packed(gmg_vec *v, double *host);
/* per-instance LRESULT of the last ls Solver on a batched hierarchy (its
 * aggregate LRESULT holds the largest defects / iteration count over the
 * instances and converged = all converged) */
int gmg_ls_instance_result(gmg_np *ls, int k, gmg_lresult *lr);

/* ------------------------------------------------ user data (udm.h) */
/* createvector: one array per level, GMG_PREC_FP64 or GMG_PREC_FP32 */
int gmg_vec_create(gmg_mg *mg, const char *name, int precision, gmg_vec **out);
gmg_vec *gmg_vec_by_name(gmg_mg *mg, const char *name);
gmg_mat *gmg_mat_by_name(gmg_mg *mg, const char *name);
/* host (UG list order, n*s doubles) <-> device, on mg's stream, synchronous */
int gmg_vec_upload(gmg_vec *v, int level, const double *host);
int gmg_vec_download(gmg_vec *v, int level, double *host);
/* device array of a level (processing order) */
int gmg_vec_device_ptr(gmg_vec *v, int level, void **ptr_dev);

/* ------------------------------------------------ numprocs (numproc.h) */
/* npcreate <objname> $c <classname>; classes: "iter.gjac", "iter.ggs",
 * "iter.gilu", "iter.glmgc", "iter.gex", "transfer.gtransfer", "linear_solver.gls" */
int gmg_np_create(gmg_mg *mg, const char *objname, const char *classname);
/* npinit <objname> <args>, e.g. "$damp 0.8", "$S pre post base $T transfer $n1 2 $n2 2 $b 2";
 * returns NP_EXECUTABLE (3), NP_ACTIVE (2) or NP_NOT_ACTIVE (1) in *status (numproc.h:54-57) */
int gmg_np_init(gmg_mg *mg, const char *objname, const char *args, int *status);
/* npexecute <objname> <args> ("$i $d $r $s $p") on the current (finest) level */
int gmg_np_execute(gmg_mg *mg, const char *objname, const char *args);
gmg_np *gmg_np_by_name(gmg_mg *mg, const char *objname);
/* Display: writes the configuration (as `npdisplay`) into buf */
int gmg_np_display(gmg_np *np, char *buf, int buflen);

/* NP_ITER (np/procs/iter.h:68-101). Iter: c <- correction, b <- b - A c. */
int gmg_iter_preprocess(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *baselevel, int *result);
int gmg_iter_iter(gmg_np *np, int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, int *result);
int gmg_iter_postprocess(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result);
/* lmgc's smoothing loop on one level (iter.cc:7811-7816 pre, 7903-7906 post):
 * `steps` times { t = Iter(b) (b -= A t); c += t }, as lmgc runs it: with
 * unit damping on a multicolour-ordered level the Gauss-Seidel steps are
 * chained (the defect stays implicit between steps, b is written once). */
int gmg_iter_smooth(gmg_np *np, int level, gmg_vec *t, gmg_vec *b, gmg_mat *A, gmg_vec *c, int steps, int *result);

/* NP_TRANSFER (np/procs/transfer.h:79-166) */
int gmg_transfer_preprocess(gmg_np *np, int *fl, int tl, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result);
int gmg_transfer_restrict_defect(gmg_np *np, int level, gmg_vec *to, gmg_vec *from, gmg_mat *A,
                                 const double *damp, int *result);
int gmg_transfer_interpolate_correction(gmg_np *np, int level, gmg_vec *to, gmg_vec *from, gmg_mat *A,
                                        const double *damp, int *result);
int gmg_transfer_postprocess(gmg_np *np, int *fl, int tl, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result);
/* NP_TRANSFER's solution operations (transfer.h:79-166 InterpolateNewVectors /
 * ProjectSolution / AdaptCorrection; transfer.cc:775, 794, 812): after a
 * refinement the new vectors (VNEW, set with gmg_mg_set_new_vectors) of levels
 * fl+1..tl take the interpolated coarse solution (StandardIntNewNodeVector,
 * transgrid.cc:354); a solution is projected from tl down to fl by copying
 * each son node's value to its father (StandardProject, transgrid.cc:655);
 * AdaptCorrection is UG's default no-op ($l is rejected). */
int gmg_transfer_interpolate_new_vectors(gmg_np *np, int fl, int tl, gmg_vec *x, int *result);
int gmg_transfer_project_solution(gmg_np *np, int fl, int tl, gmg_vec *x, int *result);
int gmg_transfer_adapt_correction(gmg_np *np, int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, int *result);
/* VNEW of a level's vectors (n ints, list order; gm.h VNEW, set for the vectors the
 * last AdaptMultiGrid created) */
int gmg_mg_set_new_vectors(gmg_mg *mg, int level, const int *vnew);
/* New matrix values of one level, structure unchanged (the next assembly of a
 * time or Newton step): val in the level's gmg_level_desc layout (list order,
 * MATRIX-list order, s*s per block).  Every device copy is rewritten in place,
 * ILU factors and the base inverse (if built) are recomputed, fused coarse
 * images and captured iteration graphs are rebuilt on next use.  Not for
 * batched hierarchies. */
int gmg_mg_update_values(gmg_mg *mg, int level, const double *val);

/* The interpolation matrix of a fine level (UG's IMATRIX: the VISTART list
 * of every VECTOR, built by AddInterpolationMatrix / CreateIMatrix,
 * np/algebra/transgrid.cc:1028, gm/algebra.cc:7601), used by a transfer
 * numproc in its matrix mode (`npinit <transfer> $M`, transfer.cc:564:
 * RestrictByMatrix / InterpolateCorrectionByMatrix, transgrid.cc:1113, 1292):
 * per VECTOR of `level` in list order (rowptr, n+1) the level-1 VECTORs it
 * couples to (col, level-1 list order) with an s*s block each (val, row-major
 * coarse component by fine component, as MVALUE of an interpolation matrix).
 * Copied; replaces an earlier one.  Not for batched hierarchies. */
int gmg_mg_set_imatrix(gmg_mg *mg, int level, const int *rowptr, const int *col, const double *val);

/* NP_LINEAR_SOLVER (np/procs/ls.h:79-132); Solver takes (abslimit, reduction)
 * in the order of np/procs/ls.cc:637. */
int gmg_ls_preprocess(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *baselevel, int *result);
int gmg_ls_defect(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result);
int gmg_ls_residuum(gmg_np *np, int fromlevel, int tolevel, gmg_vec *x, gmg_vec *b, gmg_mat *A, gmg_lresult *lr);
int gmg_ls_solver(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, const double *abslimit,
                  const double *reduction, gmg_lresult *lr);
int gmg_ls_postprocess(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result);

/* ------------------------------------------------ level kernels (ugblas.cc, ugiter.cc, transgrid.cc) */
int gmg_dset(gmg_mg *mg, int level, gmg_vec *x, double a);                              /* dset 2291 */
int gmg_dcopy(gmg_mg *mg, int level, gmg_vec *x, gmg_vec *y);                            /* dcopy: x = y */
int gmg_dadd(gmg_mg *mg, int level, gmg_vec *x, gmg_vec *y);                             /* dadd 2586: x += y */
int gmg_dmatmul_minus(gmg_mg *mg, int level, gmg_vec *x, gmg_mat *A, gmg_vec *y);        /* 3997: x -= A y */
int gmg_dnrm2x(gmg_mg *mg, int level, gmg_vec *x, double *norms);                        /* 3156 */
int gmg_dmatmul(gmg_mg *mg, int level, gmg_vec *x, gmg_mat *A, gmg_vec *y);              /* 3782: x = A y (FP64 x) */
int gmg_dmatmul_add(gmg_mg *mg, int level, gmg_vec *x, gmg_mat *A, gmg_vec *y);          /* 3889: x += A y */
int gmg_dscalx(gmg_mg *mg, int level, gmg_vec *x, const double *a);                       /* 2510: x *= a */
int gmg_daxpy(gmg_mg *mg, int level, gmg_vec *x, const double *a, gmg_vec *y);            /* 2875: x += a y */
int gmg_ddot(gmg_mg *mg, int level, gmg_vec *x, gmg_vec *y, double *result);              /* 3104 (FP64) */
int gmg_l_jac(gmg_mg *mg, int level, gmg_vec *v, gmg_mat *M, gmg_vec *d);                /* ugiter.cc:271 */
int gmg_l_lgs(gmg_mg *mg, int level, gmg_vec *v, gmg_mat *M, gmg_vec *d);                /* ugiter.cc:412 */
int gmg_l_ilu_decomp(gmg_mg *mg, int level, gmg_mat *M, const double *beta);            /* ugiter.cc:2252 */
/* the factors l_ilubthdecomp left in its copy of the matrix (decomposed on the
 * device): the level's matrix layout in processing order (gmg_mg_get_matrix),
 * diagonal blocks inverted, L below the diagonal, U above; rows that are not
 * ACTIVE keep A's values */
int gmg_l_ilu_factors(gmg_mg *mg, int level, double *lu);
int gmg_l_luiter(gmg_mg *mg, int level, gmg_vec *v, gmg_mat *M, gmg_vec *d);             /* ugiter.cc:4444 */
int gmg_standard_restrict(gmg_mg *mg, int level, gmg_vec *to, gmg_vec *from, const double *damp);            /* 462 */
int gmg_standard_interpolate_correction(gmg_mg *mg, int level, gmg_vec *to, gmg_vec *from, const double *damp); /* 529 */
/* with the level's interpolation matrix (gmg_mg_set_imatrix): transgrid.cc:1113 / 1292 */
int gmg_restrict_by_matrix(gmg_mg *mg, int level, gmg_vec *to, gmg_vec *from, const double *damp);
int gmg_interpolate_correction_by_matrix(gmg_mg *mg, int level, gmg_vec *to, gmg_vec *from, const double *damp);

/* ------------------------------------------------ allocation-free norm
 * No counterpart in the reference.  Per-component 2-norms of a device array
 * x_dev (n rows of s doubles, row-major) into norms_dev (s doubles, device),
 * for callers that cannot let a library call cudaMalloc: a host framework
 * whose memory manager owns all device memory and only hands buffers over,
 * or a process with a spent device-memory budget.  The reduction's scratch is
 * a fixed array inside the library (about 20 KB per device, held until the
 * process exits); s above GMG_MAX_S is rejected.  The first call on a device
 * looks up that array's address with the device current: make it before any
 * stream capture.  The address is kept for the life of the process: after a
 * cudaDeviceReset it is stale, so do not call this again in that process.  All calls share the array, so calls that overlap on the
 * GPU race; order them on one stream.  Enqueued on `stream` (cudaStream_t). */
int gmg_nrm2x_static(const double *x_dev, long long n, int s, double *norms_dev, void *stream);

/* ------------------------------------------------ serving pools */
/* Continuous batching of solves on resident hierarchies (no UG counterpart:
 * the request loop around UG's ls).  A pool holds `nslots` instances of one
 * cached topology -- the 3D diffusion workload's unit cube (six Kuhn
 * tetrahedra) refined `nref` (1..7) times by UG's red rules, the hierarchy
 * gmg_gen_create(3, nref, ...) builds -- as one batched hierarchy with an ls (FP32 lmgc V(2,2) with
 * `smoother` "gs" (multicolour) or "jac", base level 0, inside FP64
 * iterative refinement to `red`, at most `maxit` iterations).  A request is
 * admitted into a free slot by assembling its coefficient k = exp(g) (seed,
 * corr, var as gmg_gen_create), its matrices on every level and its
 * right-hand side on the device; each launch is one ls iteration of all
 * slots; a poll tests every active slot against its own first defect, so
 * requests join and leave between iterations (the field's precision:
 * gmg_pool_set_field_precision).  Pools run on their own
 * streams and overlap on the GPU.  Admit, fetch and slot_matrix need the
 * pool idle (the last launch polled). */
typedef struct gmg_pool gmg_pool;
int gmg_pool_create(int nref, int nslots, const char *smoother, double red, int maxit, int device, gmg_pool **out);
/* A pool whose slots hold cubes of different depths (slot k refined
 * depths[k] times, 1..7): one batched hierarchy whose level l holds level l
 * of every slot that reaches it, so one ls iteration of the pool runs the
 * V-cycles of requests of different mesh sizes together, level by level
 * (each request still iterates and converges on its own). */
int gmg_pool_create_mixed(const int *depths, int nslots, const char *smoother, double red, int maxit, int device,
                          gmg_pool **out);
/* Either of the above on a chosen mesh: `mesh` 3 = UG's red rules (what
 * gmg_pool_create / _mixed build), 1 = the Freudenthal triangulation
 * (gmg_gen_create kind 1, depths 1..9). */
int gmg_pool_create_mesh(int mesh, const int *depths, int nslots, const char *smoother, double red, int maxit,
                         int device, gmg_pool **out);
int gmg_pool_destroy(gmg_pool *pool);
gmg_mg *gmg_pool_multigrid(gmg_pool *pool);
int gmg_pool_set_stream(gmg_pool *pool, void *stream);
/* slots, VECTORs of the largest slot's finest level, free slots */
int gmg_pool_slots(const gmg_pool *pool, int *nslots, int *n_top, int *free_slots);
/* a slot's refinements and the VECTORs of its finest level */
int gmg_pool_slot_info(const gmg_pool *pool, int slot, int *nref, int *n_top);
int gmg_pool_admit(gmg_pool *pool, int slot, unsigned long long seed, double corr, double var);
/* Precision of the coefficient field at admission: GMG_PREC_FP64 (the
 * default: k within ~1e-14 of gmg_gen_create's, so a slot holds the FP64
 * problem) or GMG_PREC_FP32 (fixed-point phases and FP32 cosines, ~1e-6
 * relative in k, a cheaper admission).  Needs the pool idle. */
int gmg_pool_set_field_precision(gmg_pool *pool, int precision);
int gmg_pool_launch(gmg_pool *pool);
/* 0: still running; 1: finished, *ndone slots done (listed in done[]); -1: error */
int gmg_pool_poll(gmg_pool *pool, int *ndone, int *done);
/* a done slot's solution (n_top doubles, list order; x may be NULL) and LRESULT; frees the slot */
int gmg_pool_fetch(gmg_pool *pool, int slot, double *x, gmg_lresult *lr);
/* slot's matrix values on a level as the device holds them, in gmg_gen_levels' CSR order */
int gmg_pool_slot_matrix(gmg_pool *pool, int slot, int level, double *val);

/* ------------------------------------------------ locally refined hierarchies */
/* A hierarchy whose FINE_GRID_DOF rows (VCLASS >= 2 and VNCLASS <= 1,
 * gm/algebra.cc:2917-2921) reach below the top level is locally refined:
 * its surface spans the levels FULLREFINELEVEL..top, and ls's defect, norms
 * and update follow UG's ON_SURFACE loops (np/procs/ls.cc:562, 577, 869).
 * Host vectors of such a hierarchy hold every level, levels 0..top
 * concatenated, each in list order (as UG's VECDATA on all levels). */
int gmg_mg_full_refine_level(const gmg_mg *mg);  /* FULLREFINELEVEL (top if uniform) */
int gmg_vec_upload_levels(gmg_vec *v, const double *host);
int gmg_vec_download_levels(gmg_vec *v, double *host);

/* ------------------------------------------------ one-call solve from host buffers */
/* Uploads b (finest level, list order; packed on a batched hierarchy; every
 * level on a locally refined one), runs ls `solver` ($i $d $r $s $p, with the
 * x/b given to npinit), downloads x (same layout as b). */
int gmg_solve_host(gmg_mg *mg, const char *solver, const double *b_host, double *x_host, gmg_lresult *lr);

/* ------------------------------------------------ structured hierarchies */
/* Builds, on the host, the hierarchy UG's grid manager produces for the
 * unit square (one Q1 quad) / unit cube (six Kuhn tets) refined `nref` times
 * with `mark $a; refine`, assembled as in the workloads:
 *   kind 0: 2D Q1 Poisson;   kind 1: 3D P1 diffusion, k = exp(g) per element
 *   (exponential covariance, correlation `corr`, variance `var`; var=0 gives k=1);
 *   kind 2: 2D P1 plane-strain elasticity (E=1, nu=0.3) on two triangles, 2x2 blocks;
 *   kind 3: kind 1's problem on the cube refined by UG's red rules with the
 *   shortest interior diagonal and UG's tie-break (gm/rm.cc:1567): UG's own
 *   3D hierarchy, node for node (kind 1 refines along the diagonal that keeps
 *   the Freudenthal triangulation: same nodes and edge counts, other edges);
 *   nref <= 7.
 * Homogeneous Dirichlet boundary (unit rows, VECSKIP); the right-hand side is
 * uniform[-1,1] keyed by lattice position and `seed`, scaled by h^dim.
 * Node order per level: lexicographic.  The generator owns all arrays. */
typedef struct gmg_gen gmg_gen;
int gmg_gen_create(int kind, int nref, unsigned long long seed, double corr, double var, gmg_gen **out);
int gmg_gen_levels(gmg_gen *g, const gmg_level_desc **levels, int *nlevels);
int gmg_gen_rhs(gmg_gen *g, const double **rhs, int *len);
int gmg_gen_coords(gmg_gen *g, int level, const double **xyz);
int gmg_gen_destroy(gmg_gen *g);

/* Locally refined workload: plane-strain P1 elasticity (E=1, nu=0.3, 2x2
 * blocks) on the L-shaped domain (-1,1)^2 minus [0,1)x(-1,0], six coarse
 * triangles refined nuni times uniformly, then nloc times toward the
 * re-entrant corner (step k marks the leaf elements with a corner within
 * 0.5^k; closure, yellow copies and vector classes by UG's rules).  The
 * right-hand side holds every level, concatenated (the surface rows carry
 * the load, the others 0). */
typedef struct gmg_lgen gmg_lgen;
int gmg_lgen_create(int nuni, int nloc, unsigned long long seed, gmg_lgen **out);
int gmg_lgen_levels(gmg_lgen *g, const gmg_level_desc **levels, int *nlevels);
int gmg_lgen_rhs(gmg_lgen *g, const double **rhs, long long *len);
int gmg_lgen_coords(gmg_lgen *g, int level, const double **xyz);
int gmg_lgen_destroy(gmg_lgen *g);

/* ---- adaptation: incremental re-flattening ------------------------------
 * After AdaptMultiGrid changed the levels from_level.. (their structure,
 * values or vector classes), replace exactly those: levels[k] describes the
 * new level from_level + k (count levels, so the top may move), flattened as
 * for gmg_mg_create; the levels below from_level must be unchanged (VNCLASS of
 * a level depends on the level above it: a level whose classes changed is
 * part of the replaced range).  Kept levels keep their device arrays, factors
 * and vector values; vectors start at zero on the new levels; numprocs redo
 * their PreProcess at the next solve.  Not on batched hierarchies. */
int gmg_mg_replace_levels(gmg_mg *mg, int from_level, const gmg_level_desc *levels, int count);

/* ---- orderings: UG's order numprocs on a flattened level ----------------
 * UG orders a level's VECTOR list with its order numprocs (np/procs/order.cc:
 * order.lex, order.bw) before solving; Gauss-Seidel and ILU then visit the
 * rows in list order.  A hierarchy flattened from UG after that ordering is
 * already in the new order (GMG_ORDER_LIST follows it).  These functions
 * compute the same orders on a gmg_level_desc on the host, before
 * gmg_mg_create: perm[i] = the current index of the vector that goes to
 * position i.  The caller renumbers the level's rows and columns, P's rows on
 * this level and P's columns on the next finer level (ug_gb300.permute_levels).
 * Host work only; no device is touched. */

/* order.bw (OrderBW, order.cc:343): two breadth-first sweeps over the
 * matrix graph, the second from the vector the first reached last; entries
 * of a row in stored order.  Fails if the graph is not connected (UG
 * asserts).  bandwidth (may be NULL) = max |i - j| in the new numbering. */
int gmg_order_bw(const gmg_level_desc *level, int *perm, int *bandwidth);
/* order.lex $config <config> (OrderLex, order.cc:287 -> LexOrderVectorsInGrid,
 * gm/algebra.cc:4699): sort by position, config one letter per dimension
 * (r/l x, u/d y, f/b z; + / - direction; the last letter most significant),
 * coordinates xyz[i * xyz_stride + d], differences scaled by inv_mesh_size
 * (UG: 2^level * NN(level 0)^(1/dim) / domain radius) and equal within 1e-3. */
int gmg_order_lex(const gmg_level_desc *level, int dim, const double *xyz, int xyz_stride, const char *config,
                  double inv_mesh_size, int *perm);

#ifdef __cplusplus
}
#endif
#endif /* UG_GB300_H */
