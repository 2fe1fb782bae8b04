// Serving pools: continuous batching of lmgc solves on resident hierarchies.
//
// A pool holds `nslots` instances of one cached topology (the unit cube's
// Kuhn tetrahedra refined nref times, the 3D diffusion workload) as one
// batched hierarchy, with its ls / lmgc numprocs set up once.  A request is
// admitted into a free slot by assembling its coefficient field, matrices and
// right-hand side on the device (gmg_assemble.cu); every pool iteration is one
// batched ls iteration (a replayed CUDA graph) over all slots, in which the
// slots that are free or finished keep x unchanged.  After each iteration the
// host tests every active slot against its own first defect (the ls stopping
// rule), so requests join and leave between any two iterations: a request
// that arrives while others are iterating starts with the next iteration.
// Pools of different depths run on their own streams and overlap on the GPU.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>

#include "fields.h"
#include "gmg_internal.h"
#include "gmg_np.h"
#include "gmg_serve.h"

using namespace gmg;

enum { SLOT_FREE = 0, SLOT_ACTIVE = 1, SLOT_DONE = 2 };

struct gmg_pool {
  int nref = 0, nslots = 0, s = 1, maxit = 100;  // nref: the deepest slot's refinements
  int mesh = 3;                              // generator kind of the cubes: 3 UG's red rules, 1 Freudenthal
  std::vector<uint8_t *> masks;              // per level (UG's mesh): the tetrahedra of every cell
  double red = 1e-8, abslimit = 1e-50;
  std::vector<int> depth;                    // refinements of every slot's cube
  std::map<int, std::shared_ptr<gmg_gen>> tmpl;  // the topology of every depth (shared between pools)
  gmg_mg *mg = nullptr;
  NPLs *ls = nullptr;
  gmg_vec *x = nullptr, *b = nullptr;
  gmg_mat *A = nullptr;
  std::vector<int *> c2s;                    // per level: CSR entry -> sliced ELLPACK entry
  std::vector<int *> rows;                   // per level: the slots' rows (slot k at blk_ptr[k])
  std::vector<std::vector<SlotLevel>> sl;    // [slot][level]
  int field_prec = GMG_PREC_FP64;            // precision of the coefficient field at admission
  float *kelem = nullptr;                    // element coefficients of one level (FP32 field)
  double *kelem64 = nullptr;                 // ... (FP64 field)
  double2 *ftab = nullptr;                   // FP64 field: phase tables of one level
  double *fw_dev = nullptr, *fw_host = nullptr;  // FP64 field: w (M x 3) and phi (M) per slot
  uint32_t *prm_dev = nullptr, *prm_host = nullptr;  // FP32 field features, per slot and level
  size_t prm_stride = 0;                     // uint32 per slot
  double *first_dev = nullptr, *first_host = nullptr;
  double *norm_scratch = nullptr;            // partial sums + ticket of the admission norm
  std::vector<int> state, iters, conv, need_first;
  std::vector<double> first, last;
  cudaEvent_t ev = nullptr;
  bool inflight = false;
  int launched = 0;
  ~gmg_pool() {
    if (ev) cudaEventDestroy(ev);
    for (int *p : c2s) if (p) cudaFree(p);
    for (int *p : rows) if (p) cudaFree(p);
    for (uint8_t *p : masks) if (p) cudaFree(p);
    if (kelem) cudaFree(kelem);
    if (kelem64) cudaFree(kelem64);
    if (ftab) cudaFree(ftab);
    if (fw_dev) cudaFree(fw_dev);
    if (fw_host) cudaFreeHost(fw_host);
    if (prm_dev) cudaFree(prm_dev);
    if (prm_host) cudaFreeHost(prm_host);
    if (first_dev) cudaFree(first_dev);
    if (norm_scratch) cudaFree(norm_scratch);
    if (first_host) cudaFreeHost(first_host);
    if (mg) gmg_mg_destroy(mg);
  }
};

static int sc_less(const double *x, const double *y, int s) {  // sc_cmp, npscan.cc:1027
  for (int i = 0; i < s; ++i)
    if (std::fabs(x[i]) >= std::fabs(y[i])) return 0;
  return 1;
}

// The cube topologies of the pools, one per (mesh, depth) while any pool uses
// it: generating UG's refinement of a depth-7 cube takes seconds on the host,
// and a server holds several pools of one depth.
static std::shared_ptr<gmg_gen> topology(int mesh, int depth) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, std::weak_ptr<gmg_gen>> cache;
  std::lock_guard<std::mutex> lk(mu);
  std::weak_ptr<gmg_gen> &w = cache[{mesh, depth}];
  if (auto g = w.lock()) return g;
  gmg_gen *raw = nullptr;
  if (gmg_gen_create(mesh, depth, 0, 0.1, 0.0, &raw)) return nullptr;
  std::shared_ptr<gmg_gen> g(raw, [](gmg_gen *p) { gmg_gen_destroy(p); });
  w = g;
  return g;
}

static int np(gmg_mg *mg, const char *name, const char *cls, const char *args) {
  int st = 0;
  if (gmg_np_create(mg, name, cls) || gmg_np_init(mg, name, args, &st)) return 1;
  return 0;
}

extern "C" {

int gmg_pool_create(int nref, int nslots, const char *smoother, double red, int maxit, int device, gmg_pool **out) {
  if (nslots < 1 || nslots > (1 << 20)) {
    set_error("gmg_pool_create: bad arguments");
    return 1;
  }
  std::vector<int> d(nslots, nref);
  return gmg_pool_create_mesh(3, d.data(), nslots, smoother, red, maxit, device, out);
}

int gmg_pool_create_mixed(const int *depths, int nslots, const char *smoother, double red, int maxit, int device,
                          gmg_pool **out) {
  return gmg_pool_create_mesh(3, depths, nslots, smoother, red, maxit, device, out);
}

int gmg_pool_create_mesh(int mesh, const int *depths, int nslots, const char *smoother, double red, int maxit,
                         int device, gmg_pool **out) {
  if (!out || !depths || nslots < 1 || !smoother || (mesh != 1 && mesh != 3)) {
    set_error("gmg_pool_create: bad arguments");
    return 1;
  }
  *out = nullptr;
  const int maxd = mesh == 3 ? 7 : 9;
  for (int k = 0; k < nslots; ++k)
    GMG_CHECK(depths[k] >= 1 && depths[k] <= maxd, "gmg_pool_create: slot %d has %d refinements (1..%d)", k,
              depths[k], maxd);
  const std::string sm(smoother);
  GMG_CHECK(sm == "gs" || sm == "jac", "gmg_pool_create: smoother %s (gs or jac)", smoother);
  auto P = std::make_unique<gmg_pool>();
  P->mesh = mesh;
  P->depth.assign(depths, depths + nslots);
  const int nref = *std::max_element(depths, depths + nslots);
  P->nref = nref;
  P->nslots = nslots;
  P->red = red;
  P->maxit = maxit;
  std::vector<const gmg_level_desc *> inst(nslots);
  std::vector<int> nls(nslots);
  for (int k = 0; k < nslots; ++k) {
    std::shared_ptr<gmg_gen> &g = P->tmpl[depths[k]];
    if (!g && !(g = topology(mesh, depths[k]))) return 1;
    const gmg_level_desc *levels = nullptr;
    int nlk = 0;
    gmg_gen_levels(g.get(), &levels, &nlk);
    inst[k] = levels;
    nls[k] = nlk;
  }
  const int nl = nref + 1;
  gmg_mg_opts o{};
  o.order = GMG_ORDER_COLOR;
  o.fp32_copy = 1;
  o.device = device;
  if (gmg_mg_create_batched(inst.data(), nls.data(), nslots, &o, &P->mg)) return 1;
  gmg_mg *mg = P->mg;
  if (gmg_vec_create(mg, "sol", GMG_PREC_FP64, &P->x) || gmg_vec_create(mg, "rhs", GMG_PREC_FP64, &P->b)) return 1;
  P->A = gmg_mat_by_name(mg, "MAT");
  char args[512];
  snprintf(args, sizeof args, "$damp %s", sm == "jac" ? "0.8" : "1.0");
  // the lmgc setup of the workloads; the fused coarse cycle is off because its
  // images hold copies of the matrices, which admissions overwrite
  if (np(mg, "transfer", "transfer.gtransfer", "") || np(mg, "smooth", ("iter.g" + sm).c_str(), args) ||
      np(mg, "base", "iter.gex", "") || np(mg, "basesolver", "linear_solver.gls", "$red 1e-14 $m 1 $I base") ||
      np(mg, "lmgc", "iter.glmgc", "$S smooth smooth basesolver $T transfer $n1 2 $n2 2 $b 0 $fuse 0"))
    return 1;
  snprintf(args, sizeof args, "$A MAT $x sol $b rhs $red %.17g $abslimit 1e-50 $m %d $I lmgc $mixed 1", red, maxit);
  if (np(mg, "mgs", "linear_solver.gls", args)) return 1;
  P->ls = dynamic_cast<NPLs *>(gmg_np_by_name(mg, "mgs"));
  GMG_CHECK(P->ls, "pool: ls numproc");
  const int top = nl - 1;
  int bl = 0, res = 0;
  if (P->ls->PreProcess(top, P->x, P->b, P->A, &bl, &res) || P->ls->prepare_temps(P->b)) return 1;
  // per-level maps and slot tables; UG's mesh: every level's cells with their
  // tetrahedra (the same on every depth that reaches the level)
  P->c2s.assign(nl, nullptr);
  P->rows.assign(nl, nullptr);
  P->masks.assign(nl, nullptr);
  if (mesh == 3) {
    const gmg_gen *deep = P->tmpl[nref].get();
    for (int l = 0; l < nl; ++l) {
      const uint8_t *m = gen_cell_masks(deep, l);
      GMG_CHECK(m, "pool: no cell tetrahedra on level %d", l);
      const size_t bytes = size_t(6) << (3 * l);
      GMG_CUDA(cudaMalloc(&P->masks[l], bytes));
      GMG_CUDA(cudaMemcpy(P->masks[l], m, bytes, cudaMemcpyHostToDevice));
    }
  }
  P->sl.assign(nslots, std::vector<SlotLevel>(nl));
  for (int l = 0; l < nl; ++l) {
    Level &L = mg->lev[l];
    if (L.sell) {
      const std::vector<int> &m = L.h_sell_pos;
      GMG_CHECK((long long)m.size() == L.nnzb, "pool: sliced-ELLPACK entry map missing");
      GMG_CUDA(cudaMalloc(&P->c2s[l], m.size() * 4));
      GMG_CUDA(cudaMemcpy(P->c2s[l], m.data(), m.size() * 4, cudaMemcpyHostToDevice));
    }
    GMG_CUDA(cudaMalloc(&P->rows[l], L.blk_rows.size() * 4));
    GMG_CUDA(cudaMemcpy(P->rows[l], L.blk_rows.data(), L.blk_rows.size() * 4, cudaMemcpyHostToDevice));
    // blocks of this level: the slots that reach it, in slot order
    for (int k = 0, blk = 0; k < nslots; ++k) {
      if (P->depth[k] < l) continue;
      SlotLevel &q = P->sl[k][l];
      q.N = (1 << l) + 1;
      q.off = mg->batch.list_off[l][k];
      q.nrows = L.blk_ptr[blk + 1] - L.blk_ptr[blk];
      q.rows = P->rows[l] + L.blk_ptr[blk];
      q.masks = P->masks[l];
      ++blk;
    }
  }
  const long long nemax = 6LL << (3 * nref);
  GMG_CUDA(cudaMalloc(&P->kelem64, sizeof(double) * nemax));
  // FP64 field tables: X, Y, ZP (Nc each), three Kuhn pair factors and 27 centroid offsets per feature
  GMG_CUDA(cudaMalloc(&P->ftab, sizeof(double2) * GMG_FIELD_MAX_M * (3 * (1 << nref) + 3 + 27)));
  GMG_CUDA(cudaMalloc(&P->fw_dev, sizeof(double) * GMG_FIELD_MAX_M * 4 * nslots));
  GMG_CUDA(cudaMallocHost(&P->fw_host, sizeof(double) * GMG_FIELD_MAX_M * 4 * nslots));
  GMG_CUDA(cudaMalloc(&P->first_dev, sizeof(double) * GMG_MAX_S * nslots));
  GMG_CUDA(cudaMallocHost(&P->first_host, sizeof(double) * GMG_MAX_S * nslots));
  GMG_CUDA(cudaMalloc(&P->norm_scratch, sizeof(double) * (SLOT_NORM_BLOCKS * GMG_MAX_S + 1)));
  GMG_CUDA(cudaMemset(P->norm_scratch, 0, sizeof(double) * (SLOT_NORM_BLOCKS * GMG_MAX_S + 1)));
  GMG_CUDA(cudaEventCreateWithFlags(&P->ev, cudaEventDisableTiming));
  P->state.assign(nslots, SLOT_FREE);
  P->iters.assign(nslots, 0);
  P->conv.assign(nslots, 0);
  P->need_first.assign(nslots, 0);
  P->first.assign(size_t(nslots) * GMG_MAX_S, 0.0);
  P->last.assign(size_t(nslots) * GMG_MAX_S, 0.0);
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  *out = P.release();
  return 0;
}

int gmg_pool_destroy(gmg_pool *p) {
  if (p && p->mg) cudaStreamSynchronize(p->mg->stream);
  delete p;
  return 0;
}

gmg_mg *gmg_pool_multigrid(gmg_pool *p) { return p ? p->mg : nullptr; }

int gmg_pool_set_stream(gmg_pool *p, void *stream) {
  if (!p) return 1;
  return gmg_mg_set_stream(p->mg, stream);
}

int gmg_pool_slots(const gmg_pool *p, int *nslots, int *n_top, int *free_slots) {
  if (!p) return 1;
  if (nslots) *nslots = p->nslots;
  if (n_top) *n_top = *std::max_element(p->mg->batch.nrows_top.begin(), p->mg->batch.nrows_top.end());
  if (free_slots) *free_slots = int(std::count(p->state.begin(), p->state.end(), int(SLOT_FREE)));
  return 0;
}

int gmg_pool_slot_info(const gmg_pool *p, int k, int *nref, int *n_top) {
  if (!p || k < 0 || k >= p->nslots) { set_error("gmg_pool_slot_info: bad slot"); return 1; }
  if (nref) *nref = p->depth[k];
  if (n_top) *n_top = p->mg->batch.nrows_top[k];
  return 0;
}

// the request (seed, corr, var) into free slot k: coefficient field, matrices
// of every level, right-hand side, x = 0 and the first defect, all enqueued
int gmg_pool_admit(gmg_pool *p, int k, unsigned long long seed, double corr, double var) {
  if (!p || k < 0 || k >= p->nslots) { set_error("gmg_pool_admit: bad slot"); return 1; }
  GMG_CHECK(!p->inflight, "gmg_pool_admit: an iteration is in flight (poll first)");
  GMG_CHECK(p->state[k] == SLOT_FREE, "gmg_pool_admit: slot %d is not free", k);
  gmg_mg *mg = p->mg;
  const int nl = p->depth[k] + 1, top = p->depth[k];  // the slot's own levels
  if (p->field_prec == GMG_PREC_FP64) {
    // the field's features exactly as the host generator draws them
    int M = 0;
    double amp = 0.0;
    double *fh = p->fw_host + size_t(k) * GMG_FIELD_MAX_M * 4, *fd = p->fw_dev + size_t(k) * GMG_FIELD_MAX_M * 4;
    if (var > 0.0) {
      ugfx::LogNormalField f(seed, 3, corr, var, GMG_FIELD_MAX_M);
      M = f.M;
      amp = f.amp;
      std::memcpy(fh, f.w.data(), sizeof(double) * M * 3);
      std::memcpy(fh + GMG_FIELD_MAX_M * 3, f.phi.data(), sizeof(double) * M);
      GMG_CUDA(cudaMemcpyAsync(fd, fh, sizeof(double) * GMG_FIELD_MAX_M * 4, cudaMemcpyHostToDevice, mg->stream));
    }
    for (int l = 0; l < nl; ++l) {
      const double *ke = nullptr;
      if (var > 0.0) {
        if (k_cube_field64(mg, 1 << l, fd, fd + GMG_FIELD_MAX_M * 3, M, amp, p->ftab, p->kelem64, p->sl[k][l].masks))
          return 1;
        ke = p->kelem64;
      }
      if (k_cube_assemble64(mg, mg->lev[l], p->sl[k][l], ke, 1.0 / double(1 << l), p->c2s[l])) return 1;
    }
  } else {
    uint32_t *ph = p->prm_host + p->prm_stride * k, *pd = p->prm_dev + p->prm_stride * k;
    std::vector<float> amp(nl, 0.0f);
    std::vector<int> M(nl, 0);
    if (var > 0.0) {
      std::vector<uint32_t> prm;
      for (int l = 0; l < nl; ++l) {
        cube_field_params(seed, corr, var, l, prm, &amp[l], &M[l]);
        std::memcpy(ph + size_t(l) * GMG_FIELD_MAX_M * 4, prm.data(), prm.size() * 4);
      }
      GMG_CUDA(cudaMemcpyAsync(pd, ph, p->prm_stride * 4, cudaMemcpyHostToDevice, mg->stream));
    }
    for (int l = 0; l < nl; ++l) {
      const float *ke = nullptr;
      if (var > 0.0) {
        if (k_cube_field(mg, 1 << l, pd + size_t(l) * GMG_FIELD_MAX_M * 4, M[l], amp[l], p->kelem,
                         p->sl[k][l].masks))
          return 1;
        ke = p->kelem;
      }
      if (k_cube_assemble(mg, mg->lev[l], p->sl[k][l], ke, 1.0 / double(1 << l), p->c2s[l])) return 1;
    }
  }
  const Level &T = mg->lev[top];
  if (k_cube_rhs(mg, T, p->sl[k][top], seed, (double *)p->b->lev[top], (double *)p->x->lev[top])) return 1;
  if (k_slot_norm(mg, T, p->sl[k][top], (const double *)p->b->lev[top], p->norm_scratch,
                  p->first_dev + size_t(k) * GMG_MAX_S))
    return 1;
  GMG_CUDA(cudaMemcpyAsync(p->first_host + size_t(k) * GMG_MAX_S, p->first_dev + size_t(k) * GMG_MAX_S,
                           sizeof(double) * GMG_MAX_S, cudaMemcpyDeviceToHost, mg->stream));
  p->state[k] = SLOT_ACTIVE;
  p->iters[k] = 0;
  p->conv[k] = 0;
  p->need_first[k] = 1;
  return 0;
}

int gmg_pool_set_field_precision(gmg_pool *p, int precision) {
  if (!p || (precision != GMG_PREC_FP64 && precision != GMG_PREC_FP32)) {
    set_error("gmg_pool_set_field_precision: bad arguments");
    return 1;
  }
  GMG_CHECK(!p->inflight, "gmg_pool_set_field_precision: an iteration is in flight (poll first)");
  if (precision == GMG_PREC_FP32 && !p->kelem) {
    const int nl = p->nref + 1;
    const long long nemax = 6LL << (3 * p->nref);
    GMG_CUDA(cudaMalloc(&p->kelem, sizeof(float) * nemax));
    p->prm_stride = size_t(nl) * GMG_FIELD_MAX_M * 4;
    GMG_CUDA(cudaMalloc(&p->prm_dev, sizeof(uint32_t) * p->prm_stride * p->nslots));
    GMG_CUDA(cudaMallocHost(&p->prm_host, sizeof(uint32_t) * p->prm_stride * p->nslots));
  }
  p->field_prec = precision;
  return 0;
}

// one batched ls iteration of all active slots, enqueued (graph replay after the first)
int gmg_pool_launch(gmg_pool *p) {
  if (!p) return 1;
  GMG_CHECK(!p->inflight, "gmg_pool_launch: an iteration is in flight");
  gmg_mg *mg = p->mg;
  for (int k = 0; k < p->nslots; ++k) mg->batch.conv_host[k] = p->state[k] != SLOT_ACTIVE;
  gmg_lresult lr{};
  if (p->ls->step_async(p->launched, p->nref, p->x, p->b, p->A, &lr)) return 1;
  GMG_CUDA(cudaEventRecord(p->ev, mg->stream));
  p->inflight = true;
  p->launched++;
  return 0;
}

// 0: the iteration is still running; 1: it finished and the slots' tests ran
// (*ndone slots newly finished, listed in done[]); -1 on an error
int gmg_pool_poll(gmg_pool *p, int *ndone, int *done) {
  if (!p) return -1;
  if (ndone) *ndone = 0;
  if (!p->inflight) return 1;
  cudaError_t q = cudaEventQuery(p->ev);
  if (q == cudaErrorNotReady) return 0;
  if (q != cudaSuccess) {
    set_error("gmg_pool_poll: %s", cudaGetErrorString(q));
    return -1;
  }
  p->inflight = false;
  const int s = p->mg->lev[0].s;
  int nd = 0;
  for (int k = 0; k < p->nslots; ++k) {
    if (p->state[k] != SLOT_ACTIVE) continue;
    double *f = &p->first[size_t(k) * GMG_MAX_S], *l = &p->last[size_t(k) * GMG_MAX_S];
    if (p->need_first[k]) {
      std::memcpy(f, p->first_host + size_t(k) * GMG_MAX_S, sizeof(double) * GMG_MAX_S);
      p->need_first[k] = 0;
    }
    const double *d = p->mg->batch.norms_host + size_t(k) * GMG_MAX_S;
    p->iters[k]++;
    double reach[GMG_MAX_S], al[GMG_MAX_S];
    bool finite = true;
    for (int r = 0; r < s; ++r) {
      l[r] = d[r];
      finite = finite && std::isfinite(d[r]);
      reach[r] = f[r] * p->red;  // sc_mul_check, npscan.cc:1151
      if (reach[r] == 0.0) reach[r] = p->red;
      al[r] = p->abslimit;
    }
    const bool c = finite && (sc_less(l, al, s) || sc_less(l, reach, s));
    if (c || !finite || p->iters[k] >= p->maxit) {
      p->state[k] = SLOT_DONE;
      p->conv[k] = c;
      if (done) done[nd] = k;
      ++nd;
    }
  }
  if (ndone) *ndone = nd;
  return 1;
}

// the finished slot's solution (the instance's list order) and result; frees the slot
int gmg_pool_fetch(gmg_pool *p, int k, double *x_host, gmg_lresult *lr) {
  if (!p || k < 0 || k >= p->nslots) { set_error("gmg_pool_fetch: bad slot"); return 1; }
  GMG_CHECK(!p->inflight, "gmg_pool_fetch: an iteration is in flight (poll first)");
  GMG_CHECK(p->state[k] == SLOT_DONE, "gmg_pool_fetch: slot %d has not finished", k);
  gmg_mg *mg = p->mg;
  const auto &B = mg->batch;
  const int s = mg->lev[0].s, n = B.nrows_top[k];
  if (x_host) {
    // slot k's top level and its place in that level's instance-major lists
    const gmg_mg::Batch::TopLevel *tl = nullptr;
    int kl = -1;
    for (const auto &t : B.tops)
      for (int q = 0; q < t.ninst && kl < 0; ++q)
        if (t.ids[q] == k) { tl = &t; kl = q; }
    GMG_CHECK(tl, "gmg_pool_fetch: slot %d has no top level", k);
    std::vector<int> ptr(tl->ninst + 1);
    GMG_CUDA(cudaMemcpy(ptr.data(), tl->ptr_dev, ptr.size() * 4, cudaMemcpyDeviceToHost));
    if (k_pack_scatter_range(mg, GMG_PREC_FP64, (double *)mg->stage_dev, p->x->lev[p->depth[k]],
                             tl->rows_dev + ptr[kl], tl->pack_dev + ptr[kl], n, s))
      return 1;
    const size_t o = size_t(B.pack_off[k]) * s;
    if (stage_out(mg, x_host, o, size_t(n) * s)) return 1;
  }
  if (lr) {
    *lr = gmg_lresult{};
    lr->converged = p->conv[k];
    lr->number_of_linear_iterations = p->iters[k];
    for (int r = 0; r < s; ++r) {
      lr->first_defect[r] = p->first[size_t(k) * GMG_MAX_S + r];
      lr->last_defect[r] = p->last[size_t(k) * GMG_MAX_S + r];
    }
  }
  p->state[k] = SLOT_FREE;
  return 0;
}

// the matrix of slot k on one level as the device holds it, in the template's
// CSR order (instance list order, entries as in gmg_gen_levels)
int gmg_pool_slot_matrix(gmg_pool *p, int k, int level, double *val) {
  if (!p || k < 0 || k >= p->nslots || level < 0 || level > p->depth[k] || !val) {
    set_error("gmg_pool_slot_matrix: bad arguments");
    return 1;
  }
  gmg_mg *mg = p->mg;
  GMG_CHECK(!p->inflight, "gmg_pool_slot_matrix: an iteration is in flight");
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  const Level &L = mg->lev[level];
  std::vector<double> v(L.nnzb * L.s * L.s);
  GMG_CUDA(cudaMemcpy(v.data(), L.A.v64, v.size() * 8, cudaMemcpyDeviceToHost));
  std::vector<int> iperm(L.n);
  for (int i = 0; i < L.n; ++i) iperm[L.perm[i]] = i;
  const int off = mg->batch.list_off[level][k], n = p->sl[k][level].nrows, ss = L.s * L.s;
  size_t o = 0;
  for (int j = 0; j < n; ++j) {
    const int i = iperm[off + j];
    for (int q = L.h_rowptr[i]; q < L.h_rowptr[i + 1]; ++q, ++o)
      std::memcpy(val + o * ss, &v[size_t(q) * ss], sizeof(double) * ss);
  }
  return 0;
}

}  // extern "C"
