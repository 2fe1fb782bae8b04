// Internal data structures of the GB300 lmgc library (not part of the ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/ug_gb300.h"

namespace gmg {

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
const char *last_error();

#define GMG_CUDA(call)                                                                              \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) {                                                                        \
      ::gmg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));          \
      return 1;                                                                                     \
    }                                                                                               \
  } while (0)

#define GMG_CHECK(cond, ...)             \
  do {                                   \
    if (!(cond)) {                       \
      ::gmg::set_error(__VA_ARGS__);     \
      return 1;                          \
    }                                    \
  } while (0)

// VECTOR flags kept per row on the device (bits)
enum : uint8_t {
  F_ACTIVE = 1,  // VCLASS >= ACTIVE_CLASS (3): updated by the smoothers
  F_NEWDEF = 2,  // VCLASS >= NEWDEF_CLASS (2): restricted into the coarse grid
  F_RESET = 4,   // VNCLASS >= NEWDEF_CLASS (2): reset before restriction
  F_FINE = 8,    // FINE_GRID_DOF: VCLASS >= 2 and VNCLASS <= 1 (a surface row below the top level)
  F_VNEW = 16,   // VNEW: created by the last refinement (gmg_mg_set_new_vectors)
};

// memcpy for large host buffers (several threads)
void par_copy(void *dst, const void *src, size_t bytes);
// host vector <-> stage_dev: `n` doubles from `host` into stage_dev + off
// (queued on mg's stream; the host buffer may be reused on return), and
// stage_dev + off into `host` (returns when the copy is complete)
int stage_in(gmg_mg *mg, const double *host, size_t off, size_t n);
int stage_out(gmg_mg *mg, double *host, size_t off, size_t n);

// ---------------------------------------------------------------- device memory
// The arrays of one level live in one allocation (the level's arena);
// sub-arrays are 256-byte aligned so every row / block access can use
// 128-bit loads.
struct Arena {
  char *base = nullptr;
  size_t size = 0, used = 0;
  int alloc(size_t bytes);
  void *take(size_t bytes);
  template <class T> T *take_n(size_t n) { return static_cast<T *>(take(n * sizeof(T))); }
  void release();
};

// sparse rows on the device, one precision pair
struct DevCSR {
  int nrows = 0;
  long long nnz = 0;
  int *rowptr = nullptr, *col = nullptr;
  double *v64 = nullptr;
  float *v32 = nullptr;
};

// wavefront schedule: rows[ptr[w]..ptr[w+1]) are independent
struct Sched {
  std::vector<int> ptr;
  int *ptr_dev = nullptr;  // device copy of ptr (fused coarse cycle)
  int *rows = nullptr;
  int nwave() const { return ptr.empty() ? 0 : int(ptr.size()) - 1; }
};

// work arrays of the device ILU(0) factorisation of one level: the combined
// factor array (nnzb blocks, the level's CSR), per row its strictly lower
// entries sorted by column (lsort[lsptr[i]..lsptr[i+1]], CSR positions) and
// the smallest row whose pivot block was singular
struct IluDev {
  double *lu = nullptr;
  int *lsptr = nullptr, *lsort = nullptr, *fail = nullptr;
};

struct Level {
  Arena arena;                  // the level's device arrays (released with the level)
  int n = 0, s = 1;
  long long nnzb = 0;
  bool all_active = true;   // every row ACTIVE
  bool all_reset = true;    // every row F_RESET: a restriction into the level overwrites all of its b
  bool any_skip = false;
  // host copies in processing order
  std::vector<int> perm;       // perm[i] = UG list position of processed row i
  std::vector<int> h_rowptr, h_col;
  std::vector<double> h_val;   // blocks row-major
  std::vector<uint8_t> h_flags, h_skip;
  std::vector<int> h_prow, h_pcol;  // transfer from level-1 (processing orders)
  std::vector<double> h_pw;
  // device
  DevCSR A;                     // system matrix
  double *dinv64 = nullptr;     // inverse diagonal blocks (n*s*s)
  float *dinv32 = nullptr;
  uint8_t *flags = nullptr, *skip = nullptr;
  int *perm_dev = nullptr;
  Sched lower;                  // forward wavefronts (gs, ilu forward)
  Sched upper;                  // backward wavefronts (ilu backward)
  // ILU(0) factors in processing order (filled by the ilu numproc's PreProcess)
  bool ilu_ready = false;
  double ilu_beta[GMG_MAX_S] = {0};
  DevCSR L, U;                  // strict lower (unit diagonal) / strict upper parts
  double *udinv64 = nullptr;    // inverted diagonal blocks of U
  float *udinv32 = nullptr;
  IluDev ilu_dev;               // the device factorisation's work arrays
  std::vector<void *> own;      // cudaMalloc'd arrays owned outside the arena
  // transfer from level-1: P (rows = this level), R (rows = level-1 VECTORs)
  DevCSR P, R;
  // the level's interpolation matrix (UG's IMATRIX, gmg_mg_set_imatrix) for
  // the transfer's matrix mode: IP rows = this level's vectors, IR rows =
  // level-1 vectors (its transpose restricted to NEWDEF rows); s x s blocks,
  // coarse component major
  bool has_imat = false;
  DevCSR IP, IR;
  // son of every level-1 row: the row of this level that is its corner copy
  // (a transfer row with the single weight 1), -1 if none (StandardProject)
  int *son = nullptr;
  // base solve: explicit inverse of the level matrix (filled by ex PreProcess)
  double *ainv = nullptr;
  int base_dim = 0;
  // block-diagonal levels (batched hierarchies): rows of independent block k
  // are blk_rows[blk_ptr[k]..blk_ptr[k+1]) in processing order; the base
  // solve then keeps one dense inverse per block (at ainv + blk_aoff[k])
  std::vector<int> blk_ptr, blk_rows;
  int nblk_dev = 0;
  int *blk_ptr_dev = nullptr, *blk_rows_dev = nullptr;
  long long *blk_aoff_dev = nullptr;
  // SpMV variant: threads cooperating on one row
  int tpr = 8;
  // kernel variants of the level (autotuner; -1: by size): prefetch the
  // rows' structure before the launch wait; evict-first matrix stream
  int prefetch = -1, stream = -1;
  // chained Gauss-Seidel steps run by: 0 one launch per colour wave, 1 one
  // thread block (gs_chain_cta_ok), cw > 1 a cluster of cw blocks
  // (gs_chain_cluster_ok)
  int cta_chain = 0;
  // sliced ELLPACK copy of A (slices of 32 consecutive rows stored column by
  // column, padded to the slice's longest row with zero blocks pointing at the
  // row itself): one thread per row, coalesced 32-row loads, no reductions
  bool sell = false;
  int *sell_ptr = nullptr;  // nslices+1 entry offsets
  long long sell_nent = 0;  // stored entries (padding included)
  int sell_wmax = 0;        // entries of the widest slice's rows (diagonal included)
  int *sell_col = nullptr;
  double *sell_v64 = nullptr;
  float *sell_v32 = nullptr;
  // each row stores the diagonal, then its strictly lower blocks (sell_nl[i]
  // of them), then the upper ones; sell_split: every count fits a byte
  uint8_t *sell_nl = nullptr;
  bool sell_split = false;
  std::vector<int> h_sell_pos;  // sliced-ELLPACK entry of every CSR entry (processing order)
  // the forward schedule's wavefronts are contiguous row ranges (multicolour order)
  bool waves_contiguous = false;
  // subdomain order (GMG_ORDER_DOMAIN): rows 0..dom_nint are the interiors of
  // dom_nreg subdomains (no neighbour outside their own subdomain), the rest
  // interface rows, colour c at dom_cptr[c]..dom_cptr[c+1].  Per subdomain
  // its interior wavefronts, forward (dom_f*) and backward (dom_b*):
  // subdomain r's waves are wptr[wbeg[r]..wbeg[r+1]], wave w is rows
  // rows[wptr[w]..wptr[w+1]]; dom_iface lists rows dom_nint..n-1
  int dom_nreg = 0, dom_nint = 0;
  std::vector<int> dom_cptr;
  int *dom_fwbeg = nullptr, *dom_fwptr = nullptr, *dom_frows = nullptr;
  int *dom_bwbeg = nullptr, *dom_bwptr = nullptr, *dom_brows = nullptr;
  int *dom_iface = nullptr;
  // one-launch interface sweeps (ilu_iface_kernel): the interface rows colour
  // by colour, each colour padded to whole warps (-1 entries), forward
  // (colours 0..nc-1) and backward (nc-2..0); per-row completion flags
  // (forward, then backward) and per-direction epoch / finished-block counters
  int *iface_fw_items = nullptr, *iface_bw_items = nullptr;
  int iface_fw_n = 0, iface_bw_n = 0;
  unsigned *iface_flags = nullptr, *iface_ctr = nullptr;
  int *iface_err = nullptr;
  bool iface_coop = false;
  std::vector<int> h_dom_fwbeg, h_dom_fwptr, h_dom_frows, h_dom_bwbeg, h_dom_bwptr, h_dom_brows;
  // the ILU factors of every subdomain interior in local numbering (filled by
  // the ilu PreProcess): interior row at position p of the wave list has
  // entries ent0[p]..ent0[p+1] with the subdomain-local column col[] and the
  // factor entry k[]; a subdomain's rows outside its interior that the
  // backward sweep reads are ext[ext0[r]..ext0[r+1]] (local numbers after
  // the interior); smem = the shared memory one subdomain block needs
  struct RegionTab {
    int *ent0 = nullptr, *col = nullptr, *k = nullptr, *ext0 = nullptr, *ext = nullptr;
    int max_rows = 0, max_ent = 0, max_waves = 0;
  } dom_lt, dom_ut;
};

struct Vec {
  std::string name;
  int prec = GMG_PREC_FP64;
  std::vector<void *> lev;  // one device array per level (n*s elements)
};

struct Mat {
  std::string name;
};

// packed device image of fused coarse levels (gmg_coarse.cu), owned by the multigrid
struct CoarseImageBase {
  virtual ~CoarseImageBase() = default;
};


}  // namespace gmg

struct gmg_vec : gmg::Vec {
  gmg_mg *mg = nullptr;
};
struct gmg_mat : gmg::Mat {
  gmg_mg *mg = nullptr;
};

struct gmg_mg {
  int device = 0;
  cudaStream_t stream = nullptr;
  gmg_mg_opts opts{};
  std::vector<gmg::Level> lev;
  // FULLREFINELEVEL (gm/algebra.cc:2838): the lowest level holding a
  // FINE_GRID_DOF row; below the top level only on a locally refined
  // hierarchy, whose surface then spans levels frl..top
  int frl = 0;
  bool local() const { return frl < int(lev.size()) - 1; }
  std::map<std::string, std::unique_ptr<gmg_vec>> vecs;
  std::map<std::string, std::unique_ptr<gmg_mat>> mats;
  std::map<std::string, std::unique_ptr<gmg_np>> nps;
  bool own_stream = false;
  // scratch: reduction partials, pinned host mirror of norms, staging buffers
  double *partial = nullptr;   // GMG_REDUCE_BLOCKS * GMG_MAX_S
  double *norms_dev = nullptr; // GMG_MAX_S
  double *norms_host = nullptr;// pinned
  void *stage_dev = nullptr;   // stage_len doubles
  double *stage_host = nullptr;// pinned, stage_len doubles
  size_t stage_len = 0;        // n_top*s (every level on a locally refined hierarchy)
  // the device reads and writes pageable host memory through the host's page
  // tables (Grace: NVLink-C2C): host vectors are copied straight from / to
  // the caller's memory instead of through stage_host
  bool direct_host = false;
  // interface sweeps of the subdomain order as one cooperative launch per
  // direction (Level::iface_coop levels): 0 never (one launch per colour),
  // 1 for FP64 sweeps, 2 for both precisions.  Measured on the C3 L-shape
  // hierarchy: FP64 ILU solves 8.2 -> 10.3 /s, FP32 23.8 -> 19.8 /s (the
  // FP32 colour launches overlap through programmatic dependent launch,
  // which a cooperative launch does not)
  int iface_sweep = 1;
  long long launches = 0;
  // bumped when device copies that captured iterations point into are
  // replaced (gmg_mg_update_values drops the fused coarse images): a CUDA
  // graph captured under an older epoch is re-captured
  long long graph_epoch = 0;
  std::vector<std::unique_ptr<gmg::CoarseImageBase>> coarse_images;
  std::map<std::tuple<int, int, int, int>, long long> coarse_smem_cache;  // (bl, lc, prec, smoother)
  // batched hierarchies (gmg_mg_create_batched): independent instances stored
  // block-diagonally in every level; instance k's finest level is top[k]
  struct Batch {
    int ninst = 0;
    std::vector<int> top;                    // per instance
    std::vector<std::vector<int>> list_off;  // [level][instance] first row in list order (-1 if absent)
    std::vector<int> nrows_top;              // rows of instance k on its top level
    std::vector<long long> pack_off;         // first row of instance k in the packed layout
    // per level that is some instance's top: instances with that top (local order)
    struct TopLevel {
      int level = 0, ninst = 0, nrows = 0, nchunks = 0;
      std::vector<int> ids;                  // global instance ids
      // instance-major row lists: rows_dev[ptr_dev[k]..ptr_dev[k+1]) are the
      // rows of instance ids[k] (ascending processing order), and pack_dev[q]
      // is row q's position in the packed host layout
      int *ids_dev = nullptr, *ptr_dev = nullptr, *rows_dev = nullptr, *pack_dev = nullptr;
      // chunks of at most BATCH_CHUNK rows of one instance (host): chunk h is
      // rows chunk_q[h]..chunk_q[h+1] of instance ids[chunk_k[h]]
      std::vector<int> chunk_k, chunk_q;
    };
    std::vector<TopLevel> tops;
    // all top levels' chunks in one table (one launch per ls step): chunk h
    // is rows chunk_q0[h]..chunk_q1[h] of tops[chunk_top[h]]'s lists, of
    // instance chunk_id[h]; instance k owns chunks inst_c0[k]..inst_c1[k]
    int nchunks_all = 0;
    int *chunk_top_dev = nullptr, *chunk_id_dev = nullptr, *chunk_q0_dev = nullptr, *chunk_q1_dev = nullptr;
    int *inst_c0_dev = nullptr, *inst_c1_dev = nullptr, *ticket_dev = nullptr;
    double *partial_dev = nullptr;
    uint8_t *conv_dev = nullptr;             // converged flag per instance
    uint8_t *conv_host = nullptr;            // pinned mirror
    double *norms_dev = nullptr, *norms_host = nullptr;  // ninst * GMG_MAX_S
  } batch;
  ~gmg_mg();
};

namespace gmg {

constexpr int REDUCE_BLOCKS = 304;  // 2 x 152 SMs

// the levels of one surface operation on a locally refined hierarchy, passed
// by value to one kernel: rows row0[l]..row0[l+1] of the launch are the rows
// of table entry l; mask selects its surface rows (0: none), addx adds y to x
// on every row, b32/c32 are the FP32 copies of the mixed iteration
constexpr int SURF_MAX_LEVELS = 24;
struct SurfLevels {
  int nlev = 0;
  int row0[SURF_MAX_LEVELS + 1] = {0};
  const int *rowptr[SURF_MAX_LEVELS] = {};
  const int *col[SURF_MAX_LEVELS] = {};
  const double *val[SURF_MAX_LEVELS] = {};
  const uint8_t *flags[SURF_MAX_LEVELS] = {};
  uint8_t mask[SURF_MAX_LEVELS] = {};
  uint8_t all[SURF_MAX_LEVELS] = {};    // every row of the level (instead of mask)
  uint8_t addx[SURF_MAX_LEVELS] = {};
  double *b[SURF_MAX_LEVELS] = {};
  double *x[SURF_MAX_LEVELS] = {};
  const void *y[SURF_MAX_LEVELS] = {};
  float *b32[SURF_MAX_LEVELS] = {};
  float *c32[SURF_MAX_LEVELS] = {};
};
// selected rows (mask, or all): op 0 b -= A y, 1 b += A y, 2 b = -(A y), 3 b = A y (FP64
// matrix, y of precision yprec); addx levels: x += y on every row
int k_surf_update(gmg_mg *mg, const SurfLevels &t, int yprec, int s, int op = 0);
// dot product of x (t.b) and y (t.y) over the selected rows with the cg (kind
// 0, mode 1/2) or bcgs (kind 1, modes 0-3) scalar step on sc[], or (kind 2)
// the plain sum times sign into sc[0]
int k_surf_dot(gmg_mg *mg, const SurfLevels &t, int s, int kind, int mode, double sign, double *sc);
// b32 = b on every row; c32 = 0 where given
int k_surf_prepare(gmg_mg *mg, const SurfLevels &t, int s);
// per-component norms of b over the masked rows into mg->norms_dev
int k_surf_nrm2x(gmg_mg *mg, const SurfLevels &t, int s);
constexpr int BATCH_CHUNK = 256;    // rows per block of the batched ls update (one per thread)
#define GMG_MAX_TOPS 16             // distinct instance depths of a batched hierarchy

// ---------------------------------------------------------------- kernels (gmg_kernels.cu)
// All launchers enqueue on `st`, count launches in mg->launches, return 0 / 1.
int k_set(gmg_mg *mg, int prec, void *x, long long len, double a);
int k_copy(gmg_mg *mg, int prec, void *x, const void *y, long long len);
int k_add(gmg_mg *mg, int prec, void *x, const void *y, long long len);
int k_scale(gmg_mg *mg, int prec, void *x, int n, int s, const double *damp);
// x += a y, a per component
int k_axpy(gmg_mg *mg, int prec, void *x, const void *y, int n, int s, const double *a);
int k_convert(gmg_mg *mg, int dst_prec, void *dst, int src_prec, const void *src, long long len);
// ls's convergence loop on the device (ls.cc:680-730): one conditional WHILE
// node replays the iteration; after each pass the test counts it, keeps the
// defect norms, stops on the solver's error flag (flagged = the iteration;
// cg's (A p, p) = 0), on a non-finite norm (bad = the iteration), on
// convergence (sc_cmp against abslimit or the reduction target) or at maxit
struct LsLoopState {
  int it = 0, conv = 0, bad = 0, maxit = 0, s = 0, flagged = 0, pad[2] = {0, 0};
  double abs[GMG_MAX_S] = {0}, reach[GMG_MAX_S] = {0}, last[GMG_MAX_S] = {0};
};
// flag (device, may be null): a nonzero value ends the loop as an error
int k_ls_loop_test(gmg_mg *mg, LsLoopState *st, const double *flag, cudaGraphConditionalHandle h);
// the same on a batched hierarchy: every instance keeps its own convergence
// (batch.conv_dev), iteration count and last defect; the loop ends when all
// have converged, at maxit, or on a non-finite defect (bad_k = the lowest
// such instance, bad_it the iteration)
struct BatchLoopHead {
  int it = 0, maxit = 0, ninst = 0, s = 0, bad_k = 0, bad_it = 0, pad[2] = {0, 0};
  double abs[GMG_MAX_S] = {0};
};
int k_batch_loop_test(gmg_mg *mg, BatchLoopHead *hd, int *iters, double *last, const double *reach,
                      cudaGraphConditionalHandle h);
int k_add_mixed(gmg_mg *mg, double *x64, int src_prec, const void *c, long long len);  // x64 += c
// x -= A y (A in the precision of x/y); if acc != null also acc += y
int k_matmul_minus(gmg_mg *mg, const Level &L, int prec, void *x, const void *y, void *acc);
// FP64 x -= A64 y with y of precision yprec (iterative-refinement defect)
int k_matmul_minus_mixed(gmg_mg *mg, const Level &L, double *x, int yprec, const void *y);
// iterative-refinement update in one pass: b -= A64 c; x += c (c in FP32)
int k_refine_update(gmg_mg *mg, const Level &L, double *b, double *x, const float *c);
// t = damp * D^{-1} b on ACTIVE rows, 0 elsewhere
int k_jac(gmg_mg *mg, const Level &L, int prec, void *t, const void *b, const double *damp);
// one damped Jacobi smoothing step in one pass: t = damp D^{-1} bin (0 off
// ACTIVE rows), bout = bin - A t, c += t (bout must not alias bin)
int k_jac_step(gmg_mg *mg, const Level &L, int prec, void *bout, const void *bin, void *c, const double *damp);
// forward Gauss-Seidel in processing order over the wavefronts; t is overwritten
int k_gs(gmg_mg *mg, const Level &L, int prec, void *t, const void *b);
// `steps` multicolour Gauss-Seidel smoothing steps of lmgc (each: t = GS(b),
// c += t, b -= A t) with the defect implicit between steps; b is the final
// defect on return, t the last step's correction.  gs_chain_ok: the level
// qualifies (sliced ELLPACK, colour-contiguous waves, every row ACTIVE)
bool gs_chain_ok(const Level &L, int prec);
// want_b false: the caller never reads the final defect (lmgc's post-smoothing
// where the next restriction overwrites b), so it is not computed
int k_gs_chain(gmg_mg *mg, const Level &L, int prec, void *t, void *b, void *c, int steps, bool want_b = true);
// the chained steps of a level in one thread block (Level::cta_chain = 1):
// at most CTA_CHAIN_MAXW waves, t and c of the level in shared memory
constexpr int CTA_CHAIN_MAXW = 48;
constexpr long long CTA_CHAIN_SMEM = 200 * 1024;
struct CtaWaves {
  int n, nwave, steps;
  int own, wm;  // cluster form: slots of the block with the most rows; stored off-diagonal entries a row
  int want_b;   // write the final defect b = -U t
  int ptr[CTA_CHAIN_MAXW + 1];
};
long long gs_chain_cta_smem(const Level &L, int prec);
bool gs_chain_cta_ok(const Level &L, int prec);
// ... or in one thread-block cluster of cw = 2, 4, 8 or 16 blocks
// (Level::cta_chain = cw): every block holds all of t in shared memory
// (CLUSTER_CHAIN_SMEM with its c slots); also false where the device cannot
// co-schedule such a cluster
constexpr long long CLUSTER_CHAIN_SMEM = 227 * 1024;
long long gs_chain_cluster_smem(const Level &L, int prec, int cw);
bool gs_chain_cluster_ok(const Level &L, int prec, int cw);
// ILU forward / backward solve with the factors of L
int k_luiter(gmg_mg *mg, const Level &L, int prec, void *t, const void *b);
// ILU(0) factors of the level matrix with beta (l_ilubthdecomp) on the device,
// written into L.L / L.U / L.udinv (FP64 and FP32 copies); synchronous.
// *failed_row = the smallest processing-order row whose diagonal block was
// singular (nothing written then), else -1
int k_ilu_factor(gmg_mg *mg, Level &L, const double *beta, const IluDev &D, int *failed_row);
// RestrictByMatrix / InterpolateCorrectionByMatrix with the fine level's
// interpolation matrix (F.has_imat); zero_coarse / acc as for the standard ones
int k_restrict_imat(gmg_mg *mg, const Level &F, const Level &C, int prec, void *to, const void *from,
                    const double *damp, void *zero_coarse = nullptr);
int k_interpolate_imat(gmg_mg *mg, const Level &F, int prec, void *to, const void *from, const double *damp,
                       void *acc);
// coarse = (reset ? 0 : coarse) + R (damp*fine), honouring coarse VECSKIP
// (zero_coarse, if given, is set to 0 on the coarse level in the same pass)
int k_restrict(gmg_mg *mg, const Level &fine, const Level &coarse, int prec, void *to, const void *from,
               const double *damp, void *zero_coarse = nullptr);
// b32 = b64 and c32 = 0 in one pass (start of a mixed-precision iteration)
int k_refine_prepare(gmg_mg *mg, float *b32, float *c32, const double *b64, long long len);
// fine t = P (damp*coarse) honouring fine VECSKIP; acc += t if acc != null
int k_interpolate(gmg_mg *mg, const Level &fine, int prec, void *to, const void *from, const double *damp,
                  void *acc);
// after new matrix values (gmg_mg_update_values): the ILU factors and the
// base level's inverse of `level`, if built, recomputed into their arrays
int refresh_factors(gmg_mg *mg, int level);
// StandardIntNewNodeVector: fine rows with F_VNEW take P x_coarse (every component)
int k_interpolate_new(gmg_mg *mg, const Level &fine, int prec, void *x_fine, const void *x_coarse);
int k_interpolate_new_imat(gmg_mg *mg, const Level &fine, int prec, void *x_fine, const void *x_coarse);
// StandardProject: coarse rows with a son take the son's values
int k_project(gmg_mg *mg, const Level &fine, const Level &coarse, int prec, void *x_coarse, const void *x_fine);
// per-component 2-norms of the NEW_DEFECT rows into mg->norms_dev (device)
int k_nrm2x(gmg_mg *mg, const Level &L, int prec, const void *x);
// base level: if |b| >= abslimit in some component: t = Ainv b; b -= A t; c += t
int k_base_solve(gmg_mg *mg, const Level &L, int prec, void *c, void *b, void *t, const double *abslimit);
// batched ls, the end of an iteration over every instance's rows on its own
// finest level (all top levels, one launch): if spmv, b -= A c (FP64
// matrix); x += c unless the instance has converged (c != null); the
// per-component norms of b into batch.norms_dev[id*GMG_MAX_S + r]
int k_batch_finish(gmg_mg *mg, int bprec, gmg_vec *b, gmg_vec *x, int cprec, gmg_vec *c, bool spmv, int s);
// on every top level: b32 = b64 and c32 = 0 (one launch)
int k_batch_refine_prepare(gmg_mg *mg, gmg_vec *b32, gmg_vec *c32, gmg_vec *b64);
// on every top level: c64 = c32 (one launch)
int k_batch_widen(gmg_mg *mg, gmg_vec *c64, gmg_vec *c32);
// cg (FP64 vectors): surface dot of x and y with CGUpdate's scalar step on
// sc[] (mode 1: f = lambda/rho, rho = lambda; mode 2: alpha = rho/(sign*dot),
// sc[3] = 1 if that dot is 0); p = f p + c; x += alpha p and b += alpha tn;
// b -= t
int k_cg_dot(gmg_mg *mg, const Level &L, const double *x, const double *y, double *sc, int mode, double sign);
int k_cg_p(gmg_mg *mg, long long len, double *p, const double *c, const double *sc);
int k_cg_xb(gmg_mg *mg, long long len, double *x, const double *p, double *b, const double *tn, const double *sc);
int k_sub(gmg_mg *mg, long long len, double *b, const double *t);
// bcgs (FP64 vectors, scalars on the device in sc[]; see gmg_kernels.cu):
// ddotw with the step's scalar update (mode 0 rho, 1 alpha, 2 tt, 3 omega),
// p = beta p + b + beta omega vn, x += alpha q with s = b + alpha vn, the
// half-step test of mg->norms_dev against th, x += omega q with b = s + omega tn
int k_bcgs_dot(gmg_mg *mg, const Level &L, const double *x, const double *y, double *sc, int mode, double sign);
int k_bcgs_p(gmg_mg *mg, long long len, double *p, const double *b, const double *vn, const double *sc);
int k_bcgs_xs(gmg_mg *mg, long long len, double *x, const double *q, const double *b, double *sv, const double *vn,
              const double *sc);
int k_bcgs_half_test(gmg_mg *mg, int s, const double *th, double *sc);
int k_bcgs_xb(gmg_mg *mg, long long len, double *x, const double *q, double *b, const double *sv, const double *tn,
              const double *sc);
// the whole lmgc V-cycle (gamma = 1) over levels bl..lc in one launch of one CTA
struct CoarseCfg {
  int bl = 0, lc = 0, smoother = 0, nu1 = 1, nu2 = 1;
  int narrow = 1;  // the smallest levels by a narrow team of threads (0: the whole block)
  double damp[GMG_MAX_S], cdamp[GMG_MAX_S], abslimit[GMG_MAX_S];
};
int k_coarse_cycle(gmg_mg *mg, int prec, const CoarseCfg &cfg, gmg_vec *c, gmg_vec *b, gmg_vec *t);
// shared memory the fused cycle needs for levels bl..lc
long long coarse_smem_bytes(const gmg_mg *mg, int bl, int lc, int prec, int smoother);
constexpr long long COARSE_SMEM_BUDGET = 220 * 1024;
// default per-instance budget of the batched fused cycle (several blocks per SM)
constexpr long long BATCH_COARSE_SMEM_BUDGET = 64 * 1024;
// packed instance vectors of a batched hierarchy <-> one top level's rows
int k_pack_gather(gmg_mg *mg, int prec, void *dst, const double *packed, const gmg_mg::Batch::TopLevel &tl, int s);
int k_pack_scatter(gmg_mg *mg, int prec, double *packed, const void *src, const gmg_mg::Batch::TopLevel &tl, int s);
// the same for the m rows rows[0..m) with packed positions pack[0..m)
int k_pack_scatter_range(gmg_mg *mg, int prec, double *packed, const void *src, const int *rows, const int *pack, int m,
                         int s);
// permutations between UG list order and processing order
int k_gather(gmg_mg *mg, int prec, void *dst, const double *src_list, const int *perm, int n, int s);
int k_scatter(gmg_mg *mg, int prec, double *dst_list, const void *src, const int *perm, int n, int s);

}  // namespace gmg
