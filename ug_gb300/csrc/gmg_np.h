// Numproc classes of the GB300 lmgc path: C++ mirrors of UG's NP_BASE /
// NP_ITER / NP_TRANSFER / NP_LINEAR_SOLVER objects (np/udm/numproc.h:75-87,
// np/procs/iter.h:68-101, transfer.h:79-166, ls.h:79-132) whose methods
// enqueue CUDA kernels on the multigrid's stream instead of walking VECTOR
// lists.  Argument parsing follows npinit's `$name value` syntax.
#pragma once
#include <string>
#include <vector>

#include "gmg_internal.h"

// numproc status (np/udm/numproc.h:54-57)
enum { NP_NOT_INIT = 0, NP_NOT_ACTIVE = 1, NP_ACTIVE = 2, NP_EXECUTABLE = 3 };
enum { NPK_ITER = 1, NPK_TRANSFER = 2, NPK_LS = 3 };

namespace gmg {

// npinit / npexecute arguments: "$A MAT $x sol $red 1e-10 $i" -> {"A MAT", "x sol", "red 1e-10", "i"}
struct Args {
  std::vector<std::string> argv;
  explicit Args(const char *s);
  const std::string *find(const char *name) const;     // argument whose first word is name
  bool option(const char *name) const { return find(name) != nullptr; }
  bool get_int(const char *name, int *v) const;
  bool get_double(const char *name, double *v) const;
  bool get_word(const char *name, std::string *v) const;
  // sc_read (np/udm/npscan.cc): "$damp 0.8" (all components) or "$damp 0.8:0.5" [nd prefix allowed]
  bool get_sc(const char *name, double *v) const;
};

}  // namespace gmg

struct gmg_np {
  gmg_mg *mg = nullptr;
  std::string name, cls;
  int status = NP_NOT_INIT;
  virtual ~gmg_np() = default;
  virtual int kind() const = 0;
  virtual int Init(const gmg::Args &a) = 0;  // returns the status
  virtual std::string Display() const { return "class " + cls + "\n"; }
  virtual int Execute(const gmg::Args &a) = 0;
  // true when every call enqueues device work only (no host synchronisation),
  // so a whole cycle can be captured into a CUDA graph
  virtual bool capturable() const { return true; }
};

namespace gmg {

struct NPIter : gmg_np {
  gmg_vec *c = nullptr, *b = nullptr;
  gmg_mat *A = nullptr;
  int kind() const override { return NPK_ITER; }
  int InitIter(const Args &a);  // NPIterInit, iter.cc:674
  virtual int PreProcess(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *baselevel, int *result);
  virtual int Iter(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, int *result) = 0;
  virtual int PostProcess(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result);
  // Iter followed by acc += c (lmgc's dadd after each smoothing step);
  // smoothers fuse the addition into their defect update
  virtual int IterAcc(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, gmg_vec *acc, int *result);
  // `steps` of IterAcc in a row (lmgc's nu1 / nu2 smoothing loops); want_b
  // false: the caller never reads b afterwards, which a smoother may then
  // leave without its final defect update
  virtual int IterAccN(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, gmg_vec *acc, int steps, int *result,
                       bool want_b = true);
  int Execute(const Args &a) override;  // NPIterExecute, iter.cc:702
  std::string Display() const override;
};

// NP_SMOOTHER, iter.cc:152-177: Step, then dscalx(damp), then b -= A x
struct NPSmoother : NPIter {
  double damp[GMG_MAX_S];
  int Init(const Args &a) override;  // SmootherInit, iter.cc:763
  virtual int Step(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) = 0;
  int Iter(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, int *result) override;  // Smoother, iter.cc:817
  int IterAcc(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, gmg_vec *acc, int *result) override;
  std::string Display() const override;
};

struct NPJac : NPSmoother {  // jac, iter.cc:894-942
  int Step(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) override;
  int Iter(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, int *result) override;
  int IterAcc(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, gmg_vec *acc, int *result) override;
  // each step one fused kernel, the defect alternating between b and a scratch copy
  int IterAccN(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, gmg_vec *acc, int steps, int *result,
               bool want_b = true) override;
};

struct NPGs : NPSmoother {  // gs, iter.cc:974-1086
  int Step(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) override;
  // on colour-ordered sliced-ELLPACK levels with unit damping: the steps
  // chained, one launch per colour and step plus one for the final defect
  // (left out when the caller does not want it)
  int IterAccN(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, gmg_vec *acc, int steps, int *result,
               bool want_b = true) override;
};

struct NPIlu : NPSmoother {  // ilu, iter.cc:5383-5524
  double beta[GMG_MAX_S];
  int Init(const Args &a) override;
  int PreProcess(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *baselevel, int *result) override;
  int Step(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) override;
  std::string Display() const override;
};

struct NPEx : NPSmoother {  // ex, iter.cc:8218-9130 (exact solve on one level)
  int PreProcess(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *baselevel, int *result) override;
  int Step(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) override;
  int Iter(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, int *result) override;
};

struct NPTransfer : gmg_np {
  gmg_vec *x = nullptr, *c = nullptr, *b = nullptr;
  gmg_mat *A = nullptr;
  double damp[GMG_MAX_S];
  int baselevel = 0;
  // `$M` (IMAT_MODE, transfer.cc:564): restriction and interpolation by the
  // levels' interpolation matrices (gmg_mg_set_imatrix)
  bool imat = false;
  int kind() const override { return NPK_TRANSFER; }
  int Init(const Args &a) override;  // TransferInit + NPTransferInit, transfer.cc:553, 296
  virtual int PreProcess(int *fl, int tl, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result);
  virtual int RestrictDefect(int level, gmg_vec *to, gmg_vec *from, gmg_mat *A, const double *damp, int *result);
  virtual int InterpolateCorrection(int level, gmg_vec *to, gmg_vec *from, gmg_mat *A, const double *damp,
                                    int *result);
  virtual int PostProcess(int *fl, int tl, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result);
  // the solution on new vectors after a refinement (transfer.cc:775) and the
  // projection of a solution to the coarser levels (transfer.cc:794)
  virtual int InterpolateNewVectors(int fl, int tl, gmg_vec *x, int *result);
  virtual int ProjectSolution(int fl, int tl, gmg_vec *x, int *result);
  // transfer.cc:812: MinimizeLevel only with `$l`, which is not supported: a no-op
  virtual int AdaptCorrection(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, int *result);
  int Execute(const Args &a) override;
  std::string Display() const override;
};

struct NPLinearSolver;

struct NPLmgc : NPIter {  // lmgc, iter.cc:7578-8000
  int gamma = 1, nu1 = 1, nu2 = 1, baselevel = 0;
  NPTransfer *Transfer = nullptr;
  NPIter *PreSmooth = nullptr, *PostSmooth = nullptr;
  NPLinearSolver *BaseSolver = nullptr;
  double damp[GMG_MAX_S];
  gmg_vec *t64 = nullptr, *t32 = nullptr;  // the temporary t of Lmgc (AllocVDFromVD)
  // levels with at most fuse_rows VECTORs run as one fused kernel of one CTA
  // (gmg_coarse.cu); 0 disables
  int fuse_rows = 6000;
  // the caller of the current Iter never reads the defect it leaves on its
  // level (the parent's last coarse recursion of a V-cycle where the next
  // restriction overwrites it; the top of a uniform or batched mixed ls
  // iteration, whose FP32 defect is rebuilt from the FP64 one)
  bool defect_unused = false;
  int keep_defect = 0;  // $defect 1: every post-smoothing computes its final defect (as UG does)
  int narrow = 1;  // $narrow 0: the fused cycle runs its smallest levels with the whole block
  // batched hierarchies: the fused cycle runs one block per instance, over
  // the levels whose largest instance image fits batch_smem bytes ($bsmem; 0 disables)
  long long batch_smem = BATCH_COARSE_SMEM_BUDGET;
  bool fuse_here(int level, int prec, int smo);
  int Init(const Args &a) override;
  // smoother code of the fused kernel (0 jac, 1 gs, 2 ilu) or -1 if this
  // configuration cannot be fused
  int fusable_smoother() const;
  int PreProcess(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *baselevel, int *result) override;
  int Iter(int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, int *result) override;
  int PostProcess(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) override;
  bool capturable() const override;
  std::string Display() const override;
};

struct NPLinearSolver : gmg_np {
  gmg_vec *x = nullptr, *b = nullptr;
  gmg_mat *A = nullptr;
  double reduction[GMG_MAX_S], abslimit[GMG_MAX_S];
  int kind() const override { return NPK_LS; }
  int InitLS(const Args &a);  // NPLinearSolverInit, ls.cc:382
  virtual int PreProcess(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *baselevel, int *result) = 0;
  virtual int Defect(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) = 0;
  virtual int Residuum(int fl, int tl, gmg_vec *x, gmg_vec *b, gmg_mat *A, gmg_lresult *lr) = 0;
  virtual int Solver(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, const double *abslimit,
                     const double *reduction, gmg_lresult *lr) = 0;
  virtual int PostProcess(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) = 0;
  int Execute(const Args &a) override;  // NPLinearSolverExecute, ls.cc:436
};

// ls, np/procs/ls.cc:79-109, 539-900.  $mixed 1 runs the iteration's
// vectors in FP32 inside FP64 iterative refinement.
struct NPLs : NPLinearSolver {
  int maxiter = 0, baselevel = 0, display = 0, mixed = 0, use_graph = 1;
  NPIter *IterNp = nullptr;
  gmg_vec *cvec = nullptr;                   // correction c (precision of x, or FP32 in mixed mode)
  gmg_vec *b32 = nullptr;                    // FP32 defect in mixed mode
  gmg_vec *c64 = nullptr;                    // FP64 copy of the correction (batched mixed mode)
  bool preprocessed = false;
  // CUDA graph of one iteration (dset c; Iter; update; norm)
  cudaGraphExec_t graph = nullptr;
  int graph_level = -1;
  gmg_vec *graph_x = nullptr, *graph_b = nullptr;
  long long graph_kernels = 0;  // kernels per replay (for the launch counter)
  long long graph_epoch = 0;    // mg->graph_epoch when captured
  // the loop after the first iteration as one graph: a conditional WHILE node
  // whose body is the iteration plus the device-side test (k_ls_loop_test);
  // $dloop 0 keeps the host loop
  int use_device_loop = 1;
  bool loop_unavailable = false;  // the conditional graph failed to build: host loop
  bool norm_to_host = true;       // iteration() copies the norms to norms_host
  cudaGraphExec_t loop_graph = nullptr;
  long long loop_kernels = 0;     // kernels per pass of the body, the test included
  LsLoopState *loop_dev = nullptr, *loop_host = nullptr;
  // batched hierarchies: the per-instance loop state on the device
  BatchLoopHead *bhd_dev = nullptr, *bhd_host = nullptr;
  int *biters_dev = nullptr;
  double *blast_dev = nullptr, *breach_dev = nullptr;
  int bloop_n = 0;
  // iterations i0+1.. of batch_solver on the device; *iters = iterations run in all
  int batch_device_loop(int i0, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, const double *abslimit,
                        const std::vector<double> &reach, int *iters);
  int build_loop(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A);
  // iterations i0+1.. of Solver on the device; fills lr like the host loop
  int device_loop(int i0, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, const double *abslimit,
                  const double *reach, gmg_lresult *lr);
  ~NPLs() override;
  int Init(const Args &a) override;
  int PreProcess(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *baselevel, int *result) override;
  int Defect(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) override;
  int Residuum(int fl, int tl, gmg_vec *x, gmg_vec *b, gmg_mat *A, gmg_lresult *lr) override;
  int Solver(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, const double *abslimit, const double *reduction,
             gmg_lresult *lr) override;
  int PostProcess(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) override;
  bool capturable() const override { return false; }
  std::string Display() const override;
  // one iteration without the host-side test: dset c, Iter, update x, norm into mg->norms_dev
  virtual int iteration(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *err);
  // after every synchronised iteration: nonzero stops the solver with an error
  virtual int check_iteration(int i) { return 0; }
  // the device value check_iteration tests (null: none); on the device loop a
  // nonzero value ends the loop and check_iteration reports it
  virtual const double *iteration_flag() const { return nullptr; }
  virtual int fetch_iteration_flag() { return 0; }  // the flag's value to the host
  // the base-solver shortcut of lmgc: `ls $m 1 $I ex` as one kernel
  bool is_exact_base() const;
  // iteration i of Solver's loop (graph replay after the first), synchronised
  int step(int i, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, gmg_lresult *lr);
  int step_async(int i, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, gmg_lresult *lr);  // without the sync
  int prepare_temps(gmg_vec *b);  // the correction (and FP32 defect) vectors of Solver
  int defect_level(int level, gmg_vec *x, gmg_vec *b);
  // locally refined hierarchies: the iteration over the surface of every level
  int surface_iteration(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *err);
  // batched hierarchies (gmg_mg_create_batched), solved on their deepest level
  bool batched(int level) const;
  std::vector<double> inst_first, inst_last;  // ninst * GMG_MAX_S, per-instance defects
  std::vector<int> inst_iters, inst_conv;
  int batch_norms(gmg_vec *b);  // per-instance defect norms into batch.norms_host (async)
  int batch_iteration(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *err);
  int batch_solver(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, const double *abslimit, const double *reduction,
                   gmg_lresult *lr);
};

// cg, np/procs/ls.cc:901-1064: LinearSolver's loop with CGPrepare / CGUpdate
// (preconditioner `$I`, e.g. lmgc).  The scalars live on the device, so an
// iteration is one captured graph like ls's.  `$mixed 1` applies the
// preconditioner in FP32 (its FP64 defect is then never modified, so the
// CGUpdate step that restores it is skipped).
struct NPCg : NPLs {
  int restart = 0;
  gmg_vec *p = nullptr, *t = nullptr;
  double *sc = nullptr;       // device: f, rho, alpha, flag
  double *flag_host = nullptr;  // pinned copy of the flag
  ~NPCg() override;
  int Init(const Args &a) override;  // CGInit, ls.cc:939
  int Solver(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, const double *abslimit, const double *reduction,
             gmg_lresult *lr) override;
  int iteration(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *err) override;
  // locally refined hierarchies: CGUpdate on every level, products ON_SURFACE
  int surface_cg_iteration(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *err);
  int check_iteration(int i) override;
  const double *iteration_flag() const override { return sc + 3; }
  int fetch_iteration_flag() override;
  std::string Display() const override;
};

// bcgs, np/procs/ls.cc:1711-2062: BiCGStab preconditioned by `$I` (e.g.
// lmgc, whose multicolour Gauss-Seidel V-cycle is not symmetric), two half
// steps per iteration, each counted, with UG's stagnation test.  All scalars
// and the half-step convergence test live on the device, so an iteration is
// one captured graph; `$mixed 1` applies the preconditioner in FP32.
struct NPBcgs : NPLs {
  int restart = 0;
  gmg_vec *r = nullptr, *p = nullptr, *vn = nullptr, *sv = nullptr, *tn = nullptr, *q = nullptr, *pc = nullptr;
  double *sc = nullptr, *th = nullptr;  // device: scalars; abslimit and reduction target
  double *half_host = nullptr;          // pinned: norms of s after the first half step, then the flag
  double scal_host[3] = {1.0, 1.0, 1.0};  // restart values of alpha, rho, omega
  ~NPBcgs() override;
  int Init(const Args &a) override;  // BCGSInit, ls.cc:1750
  int Solver(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, const double *abslimit, const double *reduction,
             gmg_lresult *lr) override;
  int iteration(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *err) override;
  int precond(int level, gmg_vec *qv, gmg_vec *dv, gmg_mat *A, int *err);
  // locally refined hierarchies: every level baselevel..top, products ON_SURFACE
  int surface_bcgs_iteration(int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *err);
  int precond_levels(int level, gmg_vec *qv, gmg_vec *dv, gmg_mat *A, int *err);
  std::string Display() const override;
};

// helpers shared by the numprocs and the C ABI
gmg_vec *temp_vec(gmg_mg *mg, const std::string &name, int prec);
void *vlev(gmg_vec *v, int level);

}  // namespace gmg
