// Numprocs of the GB300 lmgc path and the C ABI around them.
//
// Each class restates the control flow of the UG numproc it mirrors (cited
// per method); the arithmetic runs in the kernels of gmg_kernels.cu on the
// multigrid's stream.  Nothing here synchronises with the device except the
// ls convergence test (one 8-byte-per-component read per iteration) and the
// explicit upload / download calls.
#include <initializer_list>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <sstream>
#include <typeinfo>

#include "gmg_internal.h"
#include "gmg_np.h"

namespace gmg {

int invert_block(int s, const double *m, double *inv);  // gmg_mg.cpp

// ------------------------------------------------------------ arguments
Args::Args(const char *s) {
  std::string cur;
  bool in = false;
  for (const char *p = s ? s : ""; *p; ++p) {
    if (*p == '$') {
      if (in) argv.push_back(cur);
      cur.clear();
      in = true;
    } else if (in && *p != ';') {
      cur += *p;
    }
  }
  if (in) argv.push_back(cur);
  for (auto &a : argv) {
    size_t b = a.find_first_not_of(" \t\n"), e = a.find_last_not_of(" \t\n");
    a = (b == std::string::npos) ? std::string() : a.substr(b, e - b + 1);
  }
}

const std::string *Args::find(const char *name) const {
  const size_t ln = strlen(name);
  for (auto &a : argv)
    if (a.compare(0, ln, name) == 0 && (a.size() == ln || a[ln] == ' ' || a[ln] == '\t')) return &a;
  return nullptr;
}

bool Args::get_int(const char *name, int *v) const {
  const std::string *a = find(name);
  if (!a) return false;
  return sscanf(a->c_str() + strlen(name), "%d", v) == 1;
}

bool Args::get_double(const char *name, double *v) const {
  const std::string *a = find(name);
  if (!a) return false;
  return sscanf(a->c_str() + strlen(name), "%lf", v) == 1;
}

bool Args::get_word(const char *name, std::string *v) const {
  const std::string *a = find(name);
  if (!a) return false;
  std::istringstream is(a->substr(strlen(name)));
  return bool(is >> *v);
}

bool Args::get_sc(const char *name, double *v) const {
  const std::string *a = find(name);
  if (!a) return false;
  std::istringstream is(a->substr(strlen(name)));
  std::string tok;
  if (!(is >> tok)) return false;
  if (tok == "nd" || tok == "ed" || tok == "el" || tok == "si")
    if (!(is >> tok)) return false;
  std::vector<double> vals;
  size_t p = 0;
  while (p <= tok.size()) {
    size_t q = tok.find(':', p);
    std::string part = tok.substr(p, q == std::string::npos ? std::string::npos : q - p);
    char *end = nullptr;
    double d = strtod(part.c_str(), &end);
    if (end == part.c_str()) return false;
    vals.push_back(d);
    if (q == std::string::npos) break;
    p = q + 1;
  }
  for (int i = 0; i < GMG_MAX_S; ++i) v[i] = vals[std::min<size_t>(i, vals.size() - 1)];
  return true;
}

// ------------------------------------------------------------ helpers
void *vlev(gmg_vec *v, int level) { return v->lev[level]; }

static gmg_vec *read_vec(gmg_mg *mg, const Args &a, const char *opt) {
  std::string n;
  if (!a.get_word(opt, &n)) return nullptr;
  auto it = mg->vecs.find(n);
  return it == mg->vecs.end() ? nullptr : it->second.get();
}
static gmg_mat *read_mat(gmg_mg *mg, const Args &a, const char *opt) {
  std::string n;
  if (!a.get_word(opt, &n)) return nullptr;
  auto it = mg->mats.find(n);
  return it == mg->mats.end() ? nullptr : it->second.get();
}
static gmg_np *read_np(gmg_mg *mg, const std::string &n, int kind) {
  auto it = mg->nps.find(n);
  if (it == mg->nps.end() || it->second->kind() != kind) return nullptr;
  return it->second.get();
}

static int alloc_vec(gmg_mg *mg, gmg_vec *v) {
  v->lev.assign(mg->lev.size(), nullptr);
  for (size_t l = 0; l < mg->lev.size(); ++l) {
    size_t len = size_t(mg->lev[l].n) * mg->lev[l].s;
    size_t bytes = (len ? len : 1) * (v->prec == GMG_PREC_FP64 ? 8 : 4);
    GMG_CUDA(cudaMalloc(&v->lev[l], bytes));
    GMG_CUDA(cudaMemsetAsync(v->lev[l], 0, bytes, mg->stream));
  }
  return 0;
}

gmg_vec *temp_vec(gmg_mg *mg, const std::string &name, int prec) {
  auto it = mg->vecs.find(name);
  if (it != mg->vecs.end()) return it->second->prec == prec ? it->second.get() : nullptr;
  auto v = std::make_unique<gmg_vec>();
  v->name = name;
  v->prec = prec;
  v->mg = mg;
  if (alloc_vec(mg, v.get())) return nullptr;
  gmg_vec *r = v.get();
  mg->vecs[name] = std::move(v);
  return r;
}

static long long vlen(gmg_mg *mg, int level) { return (long long)mg->lev[level].n * mg->lev[level].s; }

static int check_level(gmg_mg *mg, int level) {
  GMG_CHECK(level >= 0 && level < (int)mg->lev.size(), "level %d out of range", level);
  return 0;
}

static std::string fmt_sc(const double *v, int s) {
  std::ostringstream o;
  for (int i = 0; i < s; ++i) o << (i ? ":" : "") << v[i];
  return o.str();
}

// ------------------------------------------------------------ NP_ITER
int NPIter::InitIter(const Args &a) {
  A = read_mat(mg, a, "A");
  c = read_vec(mg, a, "c");
  b = read_vec(mg, a, "r");
  return (A && b && c) ? NP_EXECUTABLE : NP_ACTIVE;
}

int NPIter::PreProcess(int level, gmg_vec *, gmg_vec *, gmg_mat *, int *baselevel, int *) {
  *baselevel = level;
  return 0;
}

int NPIter::PostProcess(int, gmg_vec *, gmg_vec *, gmg_mat *, int *) { return 0; }

int NPIter::IterAcc(int level, gmg_vec *cv, gmg_vec *bv, gmg_mat *Am, gmg_vec *acc, int *result) {
  if (Iter(level, cv, bv, Am, result)) return 1;
  return k_add(mg, acc->prec, vlev(acc, level), vlev(cv, level), vlen(mg, level));
}

int NPIter::IterAccN(int level, gmg_vec *cv, gmg_vec *bv, gmg_mat *Am, gmg_vec *acc, int steps, int *result,
                     bool) {
  for (int i = 0; i < steps; ++i)
    if (IterAcc(level, cv, bv, Am, acc, result)) return 1;
  return 0;
}

// NPIterExecute, iter.cc:702-760
int NPIter::Execute(const Args &a) {
  const int level = int(mg->lev.size()) - 1;
  int result = 0, bl = 0;
  GMG_CHECK(c && b && A, "NPIterExecute: vectors c, b or matrix A missing");
  if (a.option("i") && PreProcess(level, c, b, A, &bl, &result)) return 1;
  if (a.option("s") && Iter(level, c, b, A, &result)) return 1;
  if (a.option("p") && PostProcess(level, c, b, A, &result)) return 1;
  return 0;
}

std::string NPIter::Display() const {
  std::ostringstream o;
  o << "class " << cls << "\n";
  if (A) o << "A = " << A->name << "\n";
  if (b) o << "r = " << b->name << "\n";
  if (c) o << "c = " << c->name << "\n";
  return o.str();
}

// ------------------------------------------------------------ smoothers
int NPSmoother::Init(const Args &a) {  // SmootherInit, iter.cc:763
  for (double &d : damp) d = 1.0;
  a.get_sc("damp", damp);
  return InitIter(a);
}

std::string NPSmoother::Display() const {
  return NPIter::Display() + "damp = " + fmt_sc(damp, mg->lev.empty() ? 1 : mg->lev[0].s) + "\n";
}

// Smoother, iter.cc:817-842
int NPSmoother::Iter(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *Am, int *result) {
  if (check_level(mg, level)) return 1;
  GMG_CHECK(x->prec == bv->prec, "smoother: c and b differ in precision");
  if (Step(level, x, bv, Am, result)) return 1;
  const Level &L = mg->lev[level];
  if (k_scale(mg, x->prec, vlev(x, level), L.n, L.s, damp)) return 1;
  return k_matmul_minus(mg, L, x->prec, vlev(bv, level), vlev(x, level), nullptr);
}

int NPSmoother::IterAcc(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *Am, gmg_vec *acc, int *result) {
  if (check_level(mg, level)) return 1;
  if (acc->prec != x->prec) return NPIter::IterAcc(level, x, bv, Am, acc, result);
  if (Step(level, x, bv, Am, result)) return 1;
  const Level &L = mg->lev[level];
  if (k_scale(mg, x->prec, vlev(x, level), L.n, L.s, damp)) return 1;
  return k_matmul_minus(mg, L, x->prec, vlev(bv, level), vlev(x, level), vlev(acc, level));
}

// jac: l_jac (ugiter.cc:271) with the damping folded into the same pass
int NPJac::Step(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *, int *) {
  static const double one[GMG_MAX_S] = {1, 1, 1, 1, 1, 1, 1, 1};
  return k_jac(mg, mg->lev[level], x->prec, vlev(x, level), vlev(bv, level), one);
}
int NPJac::Iter(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *, int *) {
  if (check_level(mg, level)) return 1;
  const Level &L = mg->lev[level];
  if (k_jac(mg, L, x->prec, vlev(x, level), vlev(bv, level), damp)) return 1;
  return k_matmul_minus(mg, L, x->prec, vlev(bv, level), vlev(x, level), nullptr);
}
int NPJac::IterAcc(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *Am, gmg_vec *acc, int *result) {
  if (check_level(mg, level)) return 1;
  if (acc->prec != x->prec) return NPIter::IterAcc(level, x, bv, Am, acc, result);
  const Level &L = mg->lev[level];
  if (k_jac(mg, L, x->prec, vlev(x, level), vlev(bv, level), damp)) return 1;
  return k_matmul_minus(mg, L, x->prec, vlev(bv, level), vlev(x, level), vlev(acc, level));
}

int NPJac::IterAccN(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *Am, gmg_vec *acc, int steps, int *result,
                    bool) {
  if (check_level(mg, level)) return 1;
  // FP32 only: recomputing D^{-1} b per stored entry triples the FP64
  // arithmetic per entry, and GB300's FP64 rate makes that slower than the
  // two-pass step
  if (x->prec != GMG_PREC_FP32 || acc->prec != x->prec || bv->prec != x->prec || steps < 2)
    return NPIter::IterAccN(level, x, bv, Am, acc, steps, result);
  gmg_vec *pp = temp_vec(mg, "__jac_pp" + std::to_string(x->prec), x->prec);
  GMG_CHECK(pp, "jac: temporary vector");
  const Level &L = mg->lev[level];
  void *src = vlev(bv, level), *dst = vlev(pp, level);
  for (int i = 0; i < steps; ++i) {
    if (k_jac_step(mg, L, x->prec, dst, src, vlev(acc, level), damp)) return 1;
    std::swap(src, dst);
  }
  if (src != vlev(bv, level) && k_copy(mg, x->prec, vlev(bv, level), src, vlen(mg, level))) return 1;
  return 0;
}

// gs: l_lgs (ugiter.cc:412) in the hierarchy's processing order
int NPGs::Step(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *, int *) {
  return k_gs(mg, mg->lev[level], x->prec, vlev(x, level), vlev(bv, level));
}

int NPGs::IterAccN(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *Am, gmg_vec *acc, int steps, int *result,
                   bool want_b) {
  if (check_level(mg, level)) return 1;
  const Level &L = mg->lev[level];
  bool unit = true;
  for (int r = 0; r < L.s; ++r) unit = unit && damp[r] == 1.0;
  if (!unit || steps < 2 || acc->prec != x->prec || bv->prec != x->prec || !gs_chain_ok(L, x->prec))
    return NPIter::IterAccN(level, x, bv, Am, acc, steps, result);
  return k_gs_chain(mg, L, x->prec, vlev(x, level), vlev(bv, level), vlev(acc, level), steps, want_b);
}

// ilu: ILUInit (iter.cc:5415) reads $beta (and $mindiag, unused by the decomposition)
int NPIlu::Init(const Args &a) {
  for (double &d : beta) d = 0.0;
  a.get_sc("beta", beta);
  return NPSmoother::Init(a);
}

std::string NPIlu::Display() const {
  return NPSmoother::Display() + "beta = " + fmt_sc(beta, mg->lev.empty() ? 1 : mg->lev[0].s) + "\n";
}

template <class T>
static int dev_copy(gmg::Level &L, T **dst, const std::vector<T> &src) {
  size_t n = src.empty() ? 1 : src.size();
  GMG_CUDA(cudaMalloc(dst, n * sizeof(T)));
  L.own.push_back(*dst);
  if (!src.empty()) GMG_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

static int ilu_build(gmg_mg *mg, Level &L, int level, const double *beta, bool in_place, int *result);

// the factor entries of every subdomain interior in subdomain-local numbering
// (GMG_ORDER_DOMAIN): the interior rows in wave order, then the rows outside
// the interior the sweep reads (the subdomain's own interface rows, backward
// only; the forward sweep of an interior row reads earlier interior rows only)
static int region_tables(Level &L, const std::vector<int> &wbeg, const std::vector<int> &wptr,
                         const std::vector<int> &rows, const std::vector<int> &fr, const std::vector<int> &fc, bool fwd,
                         Level::RegionTab &T) {
  std::vector<int> local(L.n, -1), ent0{0}, col, kk, ext0{0}, ext;
  T.max_rows = T.max_ent = T.max_waves = 0;
  for (int r = 0; r < L.dom_nreg; ++r) {
    const int i0 = wptr[wbeg[r]], i1 = wptr[wbeg[r + 1]], nloc = i1 - i0;
    for (int p = i0; p < i1; ++p) local[rows[p]] = p - i0;
    const size_t x0 = ext.size(), c0 = col.size();
    for (int p = i0; p < i1; ++p) {
      const int row = rows[p];
      for (int k = fr[row]; k < fr[row + 1]; ++k) {
        const int j = fc[k];
        if (local[j] < 0) {
          GMG_CHECK(!fwd, "subdomain %d: forward ILU entry outside the interior", r);
          local[j] = nloc + int(ext.size() - x0);
          ext.push_back(j);
        }
        col.push_back(local[j]);
        kk.push_back(k);
      }
      ent0.push_back(int(col.size()));
    }
    ext0.push_back(int(ext.size()));
    T.max_rows = std::max(T.max_rows, nloc + int(ext.size() - x0));
    T.max_ent = std::max(T.max_ent, int(col.size() - c0));
    T.max_waves = std::max(T.max_waves, wbeg[r + 1] - wbeg[r]);
    for (int p = i0; p < i1; ++p) local[rows[p]] = -1;
    for (size_t q = x0; q < ext.size(); ++q) local[ext[q]] = -1;
  }
  return dev_copy(L, &T.ent0, ent0) || dev_copy(L, &T.col, col) || dev_copy(L, &T.k, kk) ||
         dev_copy(L, &T.ext0, ext0) || dev_copy(L, &T.ext, ext);
}

// ILUPreProcess, iter.cc:5444: factor a copy of A and split it into the unit
// lower factor, the strict upper factor and the inverted diagonal blocks.
int NPIlu::PreProcess(int level, gmg_vec *, gmg_vec *, gmg_mat *, int *baselevel, int *result) {
  if (check_level(mg, level)) return 1;
  Level &L = mg->lev[level];
  *baselevel = level;
  if (L.ilu_ready) return 0;
  return ilu_build(mg, L, level, beta, L.L.rowptr != nullptr, result);
}

// the ILU(0) factors of level L with the given beta (l_ilubthdecomp on the
// device, gmg_ilu.cu), split into the unit lower factor, the strict upper
// factor and the inverted diagonal blocks; in_place: the level's factor
// arrays exist (same structure) and only the values are recomputed
static int ilu_build(gmg_mg *mg, Level &L, int level, const double *beta, bool in_place, int *result) {
  const int n = L.n, s = L.s, ss = s * s;
  if (!in_place) {
    // the factors' structure: active rows' strictly lower / upper entries
    // between active rows, in CSR order; per row its lower entries by column
    auto act = [&](int i) { return (L.h_flags[i] & F_ACTIVE) != 0; };
    std::vector<int> lr(n + 1, 0), ur(n + 1, 0), lc, uc, lsptr(n + 1, 0), lsort;
    std::vector<std::pair<int, int>> low;
    for (int i = 0; i < n; ++i) {
      low.clear();
      for (int k = L.h_rowptr[i]; k < L.h_rowptr[i + 1]; ++k) {
        const int j = L.h_col[k];
        if (j < i) low.push_back({j, k});
        if (j == i || !act(i) || !act(j)) continue;
        (j < i ? lc : uc).push_back(j);
      }
      std::sort(low.begin(), low.end());
      for (auto &e : low) lsort.push_back(e.second);
      lr[i + 1] = int(lc.size());
      ur[i + 1] = int(uc.size());
      lsptr[i + 1] = int(lsort.size());
    }
    // UG's MATRIX entries come in pairs (MADJ): the elimination needs (i, j)
    // wherever (j, i) is stored
    for (int i = 0; i < n; ++i)
      for (int k = L.h_rowptr[i] + 1; k < L.h_rowptr[i + 1]; ++k) {
        const int j = L.h_col[k];
        bool found = false;
        for (int q = L.h_rowptr[j]; q < L.h_rowptr[j + 1] && !found; ++q) found = L.h_col[q] == i;
        GMG_CHECK(found, "ILU: level %d: entry (%d, %d) has no transposed entry", level, L.perm[i], L.perm[j]);
      }
    auto dev_alloc = [&](auto **dst, size_t count) -> int {
      GMG_CUDA(cudaMalloc(dst, std::max<size_t>(count, 1) * sizeof(**dst)));
      L.own.push_back(*dst);
      return 0;
    };
    L.L.nrows = L.U.nrows = n;
    L.L.nnz = lc.size();
    L.U.nnz = uc.size();
    if (dev_copy(L, &L.L.rowptr, lr) || dev_copy(L, &L.L.col, lc) || dev_alloc(&L.L.v64, lc.size() * ss) ||
        dev_copy(L, &L.U.rowptr, ur) || dev_copy(L, &L.U.col, uc) || dev_alloc(&L.U.v64, uc.size() * ss) ||
        dev_alloc(&L.udinv64, size_t(n) * ss) || dev_alloc(&L.ilu_dev.lu, size_t(L.nnzb) * ss) ||
        dev_copy(L, &L.ilu_dev.lsptr, lsptr) || dev_copy(L, &L.ilu_dev.lsort, lsort) ||
        dev_alloc(&L.ilu_dev.fail, 1))
      return 1;
    if (mg->opts.fp32_copy &&
        (dev_alloc(&L.L.v32, lc.size() * ss) || dev_alloc(&L.U.v32, uc.size() * ss) ||
         dev_alloc(&L.udinv32, size_t(n) * ss)))
      return 1;
    if (L.dom_nreg > 0 &&
        (region_tables(L, L.h_dom_fwbeg, L.h_dom_fwptr, L.h_dom_frows, lr, lc, true, L.dom_lt) ||
         region_tables(L, L.h_dom_bwbeg, L.h_dom_bwptr, L.h_dom_brows, ur, uc, false, L.dom_ut)))
      return 1;
  }
  int failed = -1;
  if (k_ilu_factor(mg, L, beta, L.ilu_dev, &failed)) return 1;
  if (failed >= 0) {
    *result = -(failed + 1);
    set_error("ILU decomposition failed in row %d of level %d", failed, level);
    return 1;
  }
  std::copy(beta, beta + GMG_MAX_S, L.ilu_beta);
  L.ilu_ready = true;
  return 0;
}

int NPIlu::Step(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *, int *) {
  return k_luiter(mg, mg->lev[level], x->prec, vlev(x, level), vlev(bv, level));
}

// ex: EXPreProcess (iter.cc:8685) decomposes the level matrix once; here the
// decomposition is an explicit FP64 inverse (Gauss-Jordan, partial pivoting).
// Gauss-Jordan with partial pivoting: inv = a^{-1} (a is destroyed); returns
// 0, or the 1-based column without a pivot
static int gauss_jordan(std::vector<double> &a, std::vector<double> &inv, int N) {
  inv.assign(size_t(N) * N, 0.0);
  for (int i = 0; i < N; ++i) inv[size_t(i) * N + i] = 1.0;
  for (int c = 0; c < N; ++c) {
    int p = c;
    for (int r = c + 1; r < N; ++r)
      if (std::fabs(a[size_t(r) * N + c]) > std::fabs(a[size_t(p) * N + c])) p = r;
    if (a[size_t(p) * N + c] == 0.0) return c + 1;
    if (p != c)
      for (int k = 0; k < N; ++k) {
        std::swap(a[size_t(p) * N + k], a[size_t(c) * N + k]);
        std::swap(inv[size_t(p) * N + k], inv[size_t(c) * N + k]);
      }
    double d = 1.0 / a[size_t(c) * N + c];
    for (int k = 0; k < N; ++k) { a[size_t(c) * N + k] *= d; inv[size_t(c) * N + k] *= d; }
    for (int r = 0; r < N; ++r) {
      if (r == c) continue;
      double f = a[size_t(r) * N + c];
      if (f == 0.0) continue;
      for (int k = 0; k < N; ++k) {
        a[size_t(r) * N + k] -= f * a[size_t(c) * N + k];
        inv[size_t(r) * N + k] -= f * inv[size_t(c) * N + k];
      }
    }
  }
  return 0;
}

// dense copy of the rows `rows` (processing order, a closed block of the level)
static void dense_block(const Level &L, const int *rows, int m, std::vector<double> &a) {
  const int s = L.s, N = m * s;
  a.assign(size_t(N) * N, 0.0);
  std::map<int, int> local;
  for (int q = 0; q < m; ++q) local[rows[q]] = q;
  for (int q = 0; q < m; ++q) {
    const int i = rows[q];
    for (int k = L.h_rowptr[i]; k < L.h_rowptr[i + 1]; ++k) {
      const int j = local.at(L.h_col[k]);
      for (int r = 0; r < s; ++r)
        for (int c = 0; c < s; ++c) a[size_t(q * s + r) * N + j * s + c] = L.h_val[size_t(k) * s * s + r * s + c];
    }
  }
}

static int base_inverse(Level &L, int level, bool in_place, int *result);

int NPEx::PreProcess(int level, gmg_vec *, gmg_vec *, gmg_mat *, int *baselevel, int *result) {
  if (check_level(mg, level)) return 1;
  Level &L = mg->lev[level];
  *baselevel = level;
  if (L.ainv) return 0;
  const int s = L.s;
  std::vector<double> a, inv, all;
  if (L.blk_ptr.size() > 1) {
    // block-diagonal level of a batched hierarchy: one inverse per instance
    const int nb = int(L.blk_ptr.size()) - 1;
    std::vector<long long> aoff(nb, 0);
    for (int b = 0; b < nb; ++b) {
      const int m = L.blk_ptr[b + 1] - L.blk_ptr[b], N = m * s;
      GMG_CHECK(N <= 4096, "ex: level %d block %d has %d unknowns, above the dense base-solver limit 4096", level, b, N);
      dense_block(L, L.blk_rows.data() + L.blk_ptr[b], m, a);
      if (int c = gauss_jordan(a, inv, N)) {
        *result = -c;
        set_error("ex: singular base-level matrix of instance block %d", b);
        return 1;
      }
      aoff[b] = (long long)all.size();
      all.insert(all.end(), inv.begin(), inv.end());
    }
    GMG_CUDA(cudaMalloc(&L.ainv, std::max<size_t>(all.size(), 1) * sizeof(double)));
    GMG_CUDA(cudaMemcpy(L.ainv, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice));
    GMG_CUDA(cudaMalloc(&L.blk_ptr_dev, L.blk_ptr.size() * sizeof(int)));
    L.own.push_back(L.blk_ptr_dev);
    GMG_CUDA(cudaMemcpy(L.blk_ptr_dev, L.blk_ptr.data(), L.blk_ptr.size() * sizeof(int), cudaMemcpyHostToDevice));
    GMG_CUDA(cudaMalloc(&L.blk_rows_dev, std::max<size_t>(L.blk_rows.size(), 1) * sizeof(int)));
    L.own.push_back(L.blk_rows_dev);
    GMG_CUDA(cudaMemcpy(L.blk_rows_dev, L.blk_rows.data(), L.blk_rows.size() * sizeof(int), cudaMemcpyHostToDevice));
    GMG_CUDA(cudaMalloc(&L.blk_aoff_dev, nb * sizeof(long long)));
    L.own.push_back(L.blk_aoff_dev);
    GMG_CUDA(cudaMemcpy(L.blk_aoff_dev, aoff.data(), nb * sizeof(long long), cudaMemcpyHostToDevice));
    L.nblk_dev = nb;
    L.base_dim = 0;  // no single dense inverse (the fused coarse cycle needs one)
    return 0;
  }
  return base_inverse(L, level, false, result);
}

// the explicit inverse of a (not block-diagonal) base level; in_place: into
// the existing array (same size)
static int base_inverse(Level &L, int level, bool in_place, int *result) {
  const int N = L.n * L.s;
  GMG_CHECK(N <= 4096, "ex: level %d has %d unknowns, above the dense base-solver limit 4096", level, N);
  std::vector<double> a, inv;
  std::vector<int> rows(L.n);
  std::iota(rows.begin(), rows.end(), 0);
  dense_block(L, rows.data(), L.n, a);
  if (int c = gauss_jordan(a, inv, N)) {
    *result = -c;
    set_error("ex: singular base-level matrix");
    return 1;
  }
  if (!in_place) GMG_CUDA(cudaMalloc(&L.ainv, inv.size() * sizeof(double)));
  GMG_CUDA(cudaMemcpy(L.ainv, inv.data(), inv.size() * sizeof(double), cudaMemcpyHostToDevice));
  L.base_dim = N;
  return 0;
}

int refresh_factors(gmg_mg *mg, int level) {
  Level &L = mg->lev[level];
  int result = 0;
  if (L.ilu_ready && ilu_build(mg, L, level, L.ilu_beta, true, &result)) return 1;
  if (L.ainv && L.base_dim > 0 && base_inverse(L, level, true, &result)) return 1;
  return 0;
}

int NPEx::Step(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *Am, int *result) {
  // x = A^{-1} b without touching b: run the exact solve on a scratch defect
  gmg_vec *tb = temp_vec(mg, "__ex_b" + std::to_string(x->prec), x->prec);
  gmg_vec *tt = temp_vec(mg, "__ex_t" + std::to_string(x->prec), x->prec);
  GMG_CHECK(tb && tt, "ex: temporary vectors");
  const long long len = vlen(mg, level);
  const double never[GMG_MAX_S] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (k_copy(mg, x->prec, vlev(tb, level), vlev(bv, level), len) || k_set(mg, x->prec, vlev(x, level), len, 0.0))
    return 1;
  return k_base_solve(mg, mg->lev[level], x->prec, vlev(x, level), vlev(tb, level), vlev(tt, level), never);
}

// EXSmoother, iter.cc:8972-9068: x = A^{-1} b, x *= damp, b -= A x
int NPEx::Iter(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *Am, int *result) {
  if (check_level(mg, level)) return 1;
  bool unit = true;
  for (int r = 0; r < mg->lev[level].s; ++r) unit = unit && damp[r] == 1.0;
  if (!unit) return NPSmoother::Iter(level, x, bv, Am, result);
  gmg_vec *tt = temp_vec(mg, "__ex_t" + std::to_string(x->prec), x->prec);
  GMG_CHECK(tt, "ex: temporary vector");
  const double never[GMG_MAX_S] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (k_set(mg, x->prec, vlev(x, level), vlen(mg, level), 0.0)) return 1;
  return k_base_solve(mg, mg->lev[level], x->prec, vlev(x, level), vlev(bv, level), vlev(tt, level), never);
}

// ------------------------------------------------------------ transfer
int NPTransfer::Init(const Args &a) {  // TransferInit / NPTransferInit
  A = read_mat(mg, a, "A");
  x = read_vec(mg, a, "x");
  c = read_vec(mg, a, "c");
  b = read_vec(mg, a, "b");
  baselevel = 0;
  a.get_int("baselevel", &baselevel);
  for (double &d : damp) d = 1.0;
  a.get_sc("damp", damp);
  imat = a.option("M");
  GMG_CHECK(!a.option("R"), "transfer: $R (RestrictByMatrix_s) is not implemented");
  GMG_CHECK(!a.option("S") && !a.option("D"),
            "transfer: the scaled ($S) and Dirichlet re-assembly ($D) modes are not implemented");
  GMG_CHECK(!a.option("l"), "transfer: $l (MinimizeLevel in AdaptCorrection) is not implemented");
  return (!A && !b && !x && !c) ? NP_ACTIVE : NP_EXECUTABLE;
}

int NPTransfer::PreProcess(int *, int, gmg_vec *, gmg_vec *, gmg_mat *, int *) { return 0; }
int NPTransfer::PostProcess(int *, int, gmg_vec *, gmg_vec *, gmg_mat *, int *) { return 0; }

// RestrictDefect, transfer.cc:724: level -> level-1 with StandardRestrict
int NPTransfer::RestrictDefect(int level, gmg_vec *to, gmg_vec *from, gmg_mat *, const double *dmp, int *result) {
  if (check_level(mg, level)) return 1;
  GMG_CHECK(level >= 1, "RestrictDefect: no coarser grid below level %d", level);
  GMG_CHECK(to->prec == from->prec, "RestrictDefect: precision mismatch");
  if (imat)  // RestrictByMatrix, transgrid.cc:1113
    return k_restrict_imat(mg, mg->lev[level], mg->lev[level - 1], to->prec, vlev(to, level - 1), vlev(from, level),
                           dmp);
  return k_restrict(mg, mg->lev[level], mg->lev[level - 1], to->prec, vlev(to, level - 1), vlev(from, level), dmp);
}

// InterpolateCorrection, transfer.cc:747: level-1 -> level with StandardInterpolateCorrection
int NPTransfer::InterpolateCorrection(int level, gmg_vec *to, gmg_vec *from, gmg_mat *, const double *dmp,
                                      int *result) {
  if (check_level(mg, level)) return 1;
  GMG_CHECK(level >= 1, "InterpolateCorrection: no coarser grid below level %d", level);
  GMG_CHECK(to->prec == from->prec, "InterpolateCorrection: precision mismatch");
  if (imat)  // InterpolateCorrectionByMatrix, transgrid.cc:1292
    return k_interpolate_imat(mg, mg->lev[level], to->prec, vlev(to, level), vlev(from, level - 1), dmp, nullptr);
  return k_interpolate(mg, mg->lev[level], to->prec, vlev(to, level), vlev(from, level - 1), dmp, nullptr);
}

// InterpolateNewVectors, transfer.cc:775: the transfer's intnew on levels
// fl+1..tl -- StandardIntNewNodeVector, or InterpolateNewVectorsByMatrix
// (transgrid.cc:1425) in the matrix mode
int NPTransfer::InterpolateNewVectors(int fl, int tl, gmg_vec *xv, int *result) {
  GMG_CHECK(xv && fl >= 0 && tl < int(mg->lev.size()), "InterpolateNewVectors: bad arguments");
  for (int l = fl + 1; l <= tl; ++l) {
    const int rc = imat ? k_interpolate_new_imat(mg, mg->lev[l], xv->prec, vlev(xv, l), vlev(xv, l - 1))
                        : k_interpolate_new(mg, mg->lev[l], xv->prec, vlev(xv, l), vlev(xv, l - 1));
    if (rc) return 1;
  }
  return 0;
}

// ProjectSolution, transfer.cc:794: StandardProject on levels tl-1 down to fl
int NPTransfer::ProjectSolution(int fl, int tl, gmg_vec *xv, int *result) {
  GMG_CHECK(xv && fl >= 0 && tl < int(mg->lev.size()), "ProjectSolution: bad arguments");
  for (int l = tl - 1; l >= fl; --l)
    if (k_project(mg, mg->lev[l + 1], mg->lev[l], xv->prec, vlev(xv, l), vlev(xv, l + 1))) return 1;
  return 0;
}

int NPTransfer::AdaptCorrection(int level, gmg_vec *, gmg_vec *, gmg_mat *, int *) { return check_level(mg, level); }

int NPTransfer::Execute(const Args &a) {
  const int level = int(mg->lev.size()) - 1;
  int result = 0, fl = baselevel;
  if (a.option("i") && PreProcess(&fl, level, x, b, A, &result)) return 1;
  if (a.option("R")) {
    GMG_CHECK(b, "transfer: no vector b");
    if (RestrictDefect(level, b, b, A, damp, &result)) return 1;
  }
  if (a.option("I")) {
    GMG_CHECK(c, "transfer: no vector c");
    if (InterpolateCorrection(level, c, c, A, damp, &result)) return 1;
  }
  if (a.option("p") && PostProcess(&fl, level, x, b, A, &result)) return 1;
  return 0;
}

std::string NPTransfer::Display() const {
  if (imat)
    return "class " + cls + "\nRestrict = RestrictByMatrix\nInterpolateCor = InterpolateCorrectionByMatrix\n";
  return "class " + cls + "\nRestrict = StandardRestrict\nInterpolateCor = StandardInterpolateCorrection\n";
}

// ------------------------------------------------------------ lmgc
int NPLmgc::Init(const Args &a) {  // LmgcInit, iter.cc:7613
  std::string tn;
  Transfer = a.get_word("T", &tn) ? static_cast<NPTransfer *>(read_np(mg, tn, NPK_TRANSFER)) : nullptr;
  for (auto &arg : a.argv) {
    if (arg.empty() || arg[0] != 'S') continue;
    char pre[256], post[256], base[256];
    if (sscanf(arg.c_str(), "S %255s %255s %255s", pre, post, base) != 3) continue;
    PreSmooth = static_cast<NPIter *>(read_np(mg, pre, NPK_ITER));
    PostSmooth = static_cast<NPIter *>(read_np(mg, post, NPK_ITER));
    BaseSolver = static_cast<NPLinearSolver *>(read_np(mg, base, NPK_LS));
    break;
  }
  if (!a.get_int("g", &gamma)) gamma = 1;
  if (!a.get_int("n1", &nu1)) nu1 = 1;
  if (!a.get_int("n2", &nu2)) nu2 = 1;
  if (!a.get_int("b", &baselevel)) baselevel = 0;
  if (baselevel < 0) {  // $b -N: the finest level with at most N vectors
    int i;
    for (i = int(mg->lev.size()) - 1; i > 0; --i)
      if (mg->lev[i].n <= -baselevel) break;
    baselevel = i;
  }
  if (!a.get_int("fuse", &fuse_rows)) fuse_rows = 6000;
  if (!a.get_int("narrow", &narrow)) narrow = 1;
  if (!a.get_int("defect", &keep_defect)) keep_defect = 0;
  int bs = 0;
  batch_smem = a.get_int("bsmem", &bs) ? bs : BATCH_COARSE_SMEM_BUDGET;
  if (!Transfer || !PreSmooth || !PostSmooth || !BaseSolver) return NP_NOT_ACTIVE;
  int ret = InitIter(a);
  for (double &d : damp) d = 1.0;
  a.get_sc("damp", damp);
  return ret;
}

std::string NPLmgc::Display() const {
  std::ostringstream o;
  o << NPIter::Display() << "g = " << gamma << "\nn1 = " << nu1 << "\nn2 = " << nu2 << "\nbaselevel = " << baselevel
    << "\nfuse = " << fuse_rows << " (" << (fusable_smoother() >= 0 ? "fused coarse cycle" : "not fusable")
    << ")\nnarrow = " << narrow << "\ndefect = " << (keep_defect ? "every level" : "where read")
    << "\nT = " << (Transfer ? Transfer->name : "---") << "\npre = " << (PreSmooth ? PreSmooth->name : "---")
    << "\npost = " << (PostSmooth ? PostSmooth->name : "---") << "\nbase = " << (BaseSolver ? BaseSolver->name : "---")
    << "\n";
  return o.str();
}

int NPLmgc::fusable_smoother() const {
  if (fuse_rows <= 0 || gamma != 1 || !Transfer || !PreSmooth || !PostSmooth || !BaseSolver) return -1;
  if (typeid(*Transfer) != typeid(NPTransfer) || Transfer->imat) return -1;
  const NPLs *bls = dynamic_cast<const NPLs *>(BaseSolver);
  if (!bls || !bls->is_exact_base()) return -1;
  if (typeid(*PreSmooth) != typeid(*PostSmooth)) return -1;
  const NPSmoother *pre = dynamic_cast<const NPSmoother *>(PreSmooth);
  const NPSmoother *post = dynamic_cast<const NPSmoother *>(PostSmooth);
  for (int r = 0; r < GMG_MAX_S; ++r)
    if (pre->damp[r] != post->damp[r]) return -1;
  if (typeid(*PreSmooth) == typeid(NPJac)) return 0;
  if (typeid(*PreSmooth) == typeid(NPGs)) return 1;
  if (typeid(*PreSmooth) == typeid(NPIlu)) return 2;
  return -1;
}

bool NPLmgc::capturable() const {
  if (!Transfer || !PreSmooth || !PostSmooth || !BaseSolver) return false;
  const NPLs *bls = dynamic_cast<const NPLs *>(BaseSolver);
  bool base_ok = (bls && bls->is_exact_base()) || (gamma == 0);
  return base_ok && Transfer->capturable() && PreSmooth->capturable() && PostSmooth->capturable();
}

// LmgcPreProcess, iter.cc:7707-7739
int NPLmgc::PreProcess(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *Am, int *bl, int *result) {
  if (Transfer->PreProcess(&baselevel, level, x, bv, Am, result)) return 1;
  for (int i = baselevel + 1; i <= level; ++i)
    if (PreSmooth->PreProcess(i, x, bv, Am, bl, result)) return 1;
  if (PreSmooth != PostSmooth)
    for (int i = baselevel + 1; i <= level; ++i)
      if (PostSmooth->PreProcess(i, x, bv, Am, bl, result)) return 1;
  *bl = std::min(baselevel, level);
  if (gamma > 0 && BaseSolver->PreProcess(*bl, x, bv, Am, bl, result)) return 1;
  return 0;
}

// Lmgc, iter.cc:7741-7949
int NPLmgc::Iter(int level, gmg_vec *cv, gmg_vec *bv, gmg_mat *Am, int *result) {
  if (check_level(mg, level)) return 1;
  GMG_CHECK(cv->prec == bv->prec, "lmgc: c and b differ in precision");
  const int prec = cv->prec;
  const bool b_unused = defect_unused && !keep_defect;
  if (level <= baselevel) {
    NPLs *bls = dynamic_cast<NPLs *>(BaseSolver);
    if (bls && bls->is_exact_base()) {
      // `ls $m 1 $I ex`: one kernel with the solver's abslimit test on the device
      gmg_vec *tt = temp_vec(mg, "__lmgc_base_t" + std::to_string(prec), prec);
      GMG_CHECK(tt, "lmgc: temporary vector");
      return k_base_solve(mg, mg->lev[level], prec, vlev(cv, level), vlev(bv, level), vlev(tt, level),
                          BaseSolver->abslimit);
    }
    gmg_lresult lr{};
    if (BaseSolver->Residuum(std::min(level, baselevel), level, cv, bv, Am, &lr)) return 1;
    return BaseSolver->Solver(level, cv, bv, Am, BaseSolver->abslimit, BaseSolver->reduction, &lr);
  }
  gmg_vec *&t = prec == GMG_PREC_FP64 ? t64 : t32;
  if (!t) t = temp_vec(mg, name + "__t" + std::to_string(prec), prec);
  GMG_CHECK(t, "lmgc: temporary vector");
  const int smo = fusable_smoother();
  if (smo >= 0 && fuse_here(level, prec, smo)) {
    // this level and everything below it: one fused kernel (a single CTA)
    CoarseCfg cfg;
    cfg.bl = baselevel; cfg.lc = level; cfg.smoother = smo;
    cfg.nu1 = nu1; cfg.nu2 = nu2; cfg.narrow = narrow;
    const NPSmoother *sm = static_cast<const NPSmoother *>(PreSmooth);
    for (int r = 0; r < GMG_MAX_S; ++r) {
      cfg.damp[r] = sm->damp[r];
      cfg.cdamp[r] = damp[r];
      cfg.abslimit[r] = BaseSolver->abslimit[r];
    }
    return k_coarse_cycle(mg, prec, cfg, cv, bv, t);
  }
  if (PreSmooth->IterAccN(level, t, bv, Am, cv, nu1, result)) return 1;
  static const double one[GMG_MAX_S] = {1, 1, 1, 1, 1, 1, 1, 1};  // Factor_One
  if (typeid(*Transfer) == typeid(NPTransfer)) {
    // StandardRestrict (or RestrictByMatrix) and dset(c_{l-1}, 0) in one pass
    if (Transfer->imat ? k_restrict_imat(mg, mg->lev[level], mg->lev[level - 1], prec, vlev(bv, level - 1),
                                         vlev(bv, level), one, vlev(cv, level - 1))
                       : k_restrict(mg, mg->lev[level], mg->lev[level - 1], prec, vlev(bv, level - 1),
                                    vlev(bv, level), one, vlev(cv, level - 1)))
      return 1;
  } else {
    if (Transfer->RestrictDefect(level, bv, bv, Am, one, result)) return 1;
    if (k_set(mg, prec, vlev(cv, level - 1), vlen(mg, level - 1), 0.0)) return 1;
  }
  // the defect the last coarse recursion leaves is never read when the next
  // restriction overwrites all of it (StandardRestrict onto rows that all
  // reset, not surface-based; a batched level that is some instance's top
  // keeps that instance's rows, VNCLASS < 2, so it never qualifies): its
  // post-smoothing may skip it
  const bool coarse_b_dead = !keep_defect && typeid(*Transfer) == typeid(NPTransfer) && !Transfer->imat &&
                             !mg->local() && mg->lev[level - 1].all_reset;
  for (int i = 0; i < gamma; ++i) {
    defect_unused = coarse_b_dead && i == gamma - 1;
    const int rc = Iter(level - 1, cv, bv, Am, result);
    defect_unused = b_unused;
    if (rc) return 1;
  }
  // t = P c_{l-1} * damp; c += t (fused); b -= A t
  if (dynamic_cast<NPTransfer *>(Transfer) && typeid(*Transfer) == typeid(NPTransfer)) {
    if (Transfer->imat ? k_interpolate_imat(mg, mg->lev[level], prec, vlev(t, level), vlev(cv, level - 1), damp,
                                            vlev(cv, level))
                       : k_interpolate(mg, mg->lev[level], prec, vlev(t, level), vlev(cv, level - 1), damp,
                                       vlev(cv, level)))
      return 1;
  } else {
    if (Transfer->InterpolateCorrection(level, t, cv, Am, damp, result)) return 1;
    if (k_add(mg, prec, vlev(cv, level), vlev(t, level), vlen(mg, level))) return 1;
  }
  if (k_matmul_minus(mg, mg->lev[level], prec, vlev(bv, level), vlev(t, level), nullptr)) return 1;
  if (PostSmooth->IterAccN(level, t, bv, Am, cv, nu2, result, !b_unused)) return 1;
  return 0;
}

bool NPLmgc::fuse_here(int level, int prec, int smo) {
  if (mg->batch.ninst == 0)
    return mg->lev[level].n <= fuse_rows && coarse_smem_bytes(mg, baselevel, level, prec, smo) <= COARSE_SMEM_BUDGET;
  return batch_smem > 0 && fuse_rows > 0 && coarse_smem_bytes(mg, baselevel, level, prec, smo) <= batch_smem;
}

// LmgcPostProcess, iter.cc:7951
int NPLmgc::PostProcess(int level, gmg_vec *x, gmg_vec *bv, gmg_mat *Am, int *result) {
  if (gamma > 0 && BaseSolver->PostProcess(baselevel, x, bv, Am, result)) return 1;
  if (PreSmooth != PostSmooth)
    for (int i = level; i >= baselevel + 1; --i)
      if (PostSmooth->PostProcess(i, x, bv, Am, result)) return 1;
  for (int i = level; i >= baselevel + 1; --i)
    if (PreSmooth->PostProcess(i, x, bv, Am, result)) return 1;
  int fl = baselevel;
  return Transfer->PostProcess(&fl, level, x, bv, Am, result);
}

// ------------------------------------------------------------ linear solver
int NPLinearSolver::InitLS(const Args &a) {  // NPLinearSolverInit, ls.cc:382
  A = read_mat(mg, a, "A");
  x = read_vec(mg, a, "x");
  b = read_vec(mg, a, "b");
  if (!a.get_sc("abslimit", abslimit))
    for (double &d : abslimit) d = 1e-10;  // ABS_LIMIT, ls.cc:66
  if (!a.get_sc("red", reduction)) return NP_ACTIVE;
  if (!x || !b || !A) return NP_ACTIVE;
  return NP_EXECUTABLE;
}

// NPLinearSolverExecute, ls.cc:436-537
int NPLinearSolver::Execute(const Args &a) {
  const int level = int(mg->lev.size()) - 1;
  int result = 0, bl = 0;
  GMG_CHECK(x && b && A, "NPLinearSolverExecute: x, b or A missing");
  gmg_lresult lr{};
  if (a.option("i") && PreProcess(level, x, b, A, &bl, &result)) return 1;
  if (a.option("d") && Defect(level, x, b, A, &result)) return 1;
  if (a.option("r") && Residuum(bl, level, x, b, A, &lr)) return 1;
  if (a.option("s") && Solver(level, x, b, A, abslimit, reduction, &lr)) return 1;
  if (a.option("p") && PostProcess(level, x, b, A, &result)) return 1;
  return 0;
}

NPLs::~NPLs() {
  if (graph) cudaGraphExecDestroy(graph);
  if (loop_graph) cudaGraphExecDestroy(loop_graph);
  if (loop_dev) cudaFree(loop_dev);
  if (loop_host) cudaFreeHost(loop_host);
  if (bhd_dev) cudaFree(bhd_dev);
  if (bhd_host) cudaFreeHost(bhd_host);
  if (biters_dev) cudaFree(biters_dev);
  if (blast_dev) cudaFree(blast_dev);
  if (breach_dev) cudaFree(breach_dev);
}

int NPLs::Init(const Args &a) {  // LinearSolverInit, ls.cc:788
  if (!a.get_int("m", &maxiter)) return NP_NOT_ACTIVE;
  std::string itn;
  IterNp = a.get_word("I", &itn) ? static_cast<NPIter *>(read_np(mg, itn, NPK_ITER)) : nullptr;
  if (!IterNp) return NP_NOT_ACTIVE;
  baselevel = 0;
  cvec = read_vec(mg, a, "c");
  std::string d;
  display = a.get_word("d", &d) ? (d == "full" ? 2 : d == "red" ? 1 : 0) : 0;
  if (!a.get_int("mixed", &mixed)) mixed = 0;
  if (!a.get_int("graph", &use_graph)) use_graph = 1;
  if (!a.get_int("dloop", &use_device_loop)) use_device_loop = 1;
  if (graph) { cudaGraphExecDestroy(graph); graph = nullptr; }
  if (loop_graph) { cudaGraphExecDestroy(loop_graph); loop_graph = nullptr; }
  return InitLS(a);
}

std::string NPLs::Display() const {
  std::ostringstream o;
  o << "class " << cls << "\nm = " << maxiter << "\nbaselevel = " << baselevel
    << "\nIter = " << (IterNp ? IterNp->name : "---") << "\nmixed = " << mixed << "\nloop = "
    << (!use_device_loop || !use_graph ? "host" : loop_unavailable ? "host (conditional graph unavailable)"
                                                                   : loop_graph ? "device (built)" : "device")
    << "\nred = "
    << fmt_sc(reduction, 1) << "\nabslimit = " << fmt_sc(abslimit, 1) << "\n";
  return o.str();
}

bool NPLs::is_exact_base() const {
  if (maxiter != 1 || !IterNp) return false;
  const NPEx *ex = dynamic_cast<const NPEx *>(IterNp);
  if (!ex) return false;
  for (int r = 0; r < GMG_MAX_S; ++r)
    if (ex->damp[r] != 1.0) return false;
  return true;
}

// LinearSolverPreProcess, ls.cc:539
int NPLs::PreProcess(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, int *bl, int *result) {
  if (IterNp->PreProcess(level, xv, bv, Am, bl, result)) return 1;
  baselevel = std::min(*bl, level);
  preprocessed = true;
  return 0;
}

bool NPLs::batched(int level) const { return mg->batch.ninst > 0 && level == int(mg->lev.size()) - 1; }

// ---- the surface of a locally refined hierarchy
// ON_SURFACE with tolevel tl (np/algebra/vecloop.ct, matloop.ct): the
// FINE_GRID_DOF rows of the levels FULLREFINELEVEL..tl-1 and the NEW_DEFECT
// rows of tl.  Table entries for the levels lo..hi, with that row mask on the
// levels from FULLREFINELEVEL up (none below).
static void surf_table(gmg_mg *mg, int lo, int hi, int tl, SurfLevels &t) {
  t = SurfLevels{};
  for (int l = lo; l <= hi; ++l) {
    const Level &L = mg->lev[l];
    const int e = t.nlev++;
    t.row0[e + 1] = t.row0[e] + L.n;
    t.rowptr[e] = L.A.rowptr; t.col[e] = L.A.col; t.val[e] = L.A.v64; t.flags[e] = L.flags;
    t.mask[e] = l == tl ? F_NEWDEF : (l >= mg->frl && l < tl ? F_FINE : 0);
  }
}

static int surf_lo(gmg_mg *mg, int tl) { return std::min(mg->frl, tl); }

// LinearDefect ON_SURFACE: b -= A x on the surface rows, level by level
static int surface_defect(gmg_mg *mg, int tl, gmg_vec *xv, gmg_vec *bv) {
  GMG_CHECK(bv->prec == GMG_PREC_FP64, "ls: a locally refined hierarchy needs an FP64 defect");
  SurfLevels t;
  surf_table(mg, surf_lo(mg, tl), tl, tl, t);
  for (int e = 0; e < t.nlev; ++e) {
    const int l = surf_lo(mg, tl) + e;
    t.b[e] = (double *)vlev(bv, l);
    t.y[e] = vlev(xv, l);
  }
  return k_surf_update(mg, t, xv->prec, mg->lev[tl].s);
}

// dnrm2x ON_SURFACE into mg->norms_dev
static int surface_norm(gmg_mg *mg, int tl, gmg_vec *bv) {
  GMG_CHECK(bv->prec == GMG_PREC_FP64, "ls: a locally refined hierarchy needs an FP64 defect");
  SurfLevels t;
  surf_table(mg, surf_lo(mg, tl), tl, tl, t);
  for (int e = 0; e < t.nlev; ++e) t.b[e] = (double *)vlev(bv, surf_lo(mg, tl) + e);
  return k_surf_nrm2x(mg, t, mg->lev[tl].s);
}

// LinearDefect, ls.cc:562: b -= A x on the surface, which is the top level
// of a uniformly refined hierarchy (on a batched hierarchy: every instance's
// own top level; a level that is some instance's top is updated whole, which
// only touches the other instances' restricted, reset rows there)
int NPLs::Defect(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, int *res) {
  if (check_level(mg, level)) return 1;
  if (mg->local()) return surface_defect(mg, level, xv, bv);
  if (batched(level)) {
    for (const auto &tl : mg->batch.tops)
      if (defect_level(tl.level, xv, bv)) return 1;
    return 0;
  }
  return defect_level(level, xv, bv);
}

int NPLs::defect_level(int level, gmg_vec *xv, gmg_vec *bv) {
  if (bv->prec == GMG_PREC_FP64)
    return k_matmul_minus_mixed(mg, mg->lev[level], (double *)vlev(bv, level), xv->prec, vlev(xv, level));
  GMG_CHECK(xv->prec == bv->prec, "ls: precision mismatch");
  return k_matmul_minus(mg, mg->lev[level], bv->prec, vlev(bv, level), vlev(xv, level), nullptr);
}

// LinearResiduum, ls.cc:577: per-component norms of b
int NPLs::Residuum(int, int tl, gmg_vec *, gmg_vec *bv, gmg_mat *, gmg_lresult *lr) {
  if (check_level(mg, tl)) return 1;
  const int s = mg->lev[tl].s;
  if (batched(tl)) {
    // per-instance defect norms, each on the instance's own top level
    const auto &B = mg->batch;
    if (batch_norms(bv)) return 1;
    GMG_CUDA(cudaStreamSynchronize(mg->stream));
    inst_last.assign(B.norms_host, B.norms_host + size_t(B.ninst) * GMG_MAX_S);
    for (int r = 0; r < s; ++r) {
      lr->last_defect[r] = 0.0;
      for (int k = 0; k < B.ninst; ++k) lr->last_defect[r] = std::max(lr->last_defect[r], inst_last[k * GMG_MAX_S + r]);
    }
    return 0;
  }
  if (mg->local() ? surface_norm(mg, tl, bv) : k_nrm2x(mg, mg->lev[tl], bv->prec, vlev(bv, tl))) return 1;
  GMG_CUDA(cudaMemcpyAsync(mg->norms_host, mg->norms_dev, sizeof(double) * s, cudaMemcpyDeviceToHost, mg->stream));
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  for (int r = 0; r < s; ++r) lr->last_defect[r] = mg->norms_host[r];
  return 0;
}

// one ls iteration on a locally refined hierarchy.  LSUpdate adds c on every
// level baselevel..top (ls.cc:869); lmgc has kept the surface defect on the
// FINE_GRID_DOF rows of the lower levels (restriction resets only VNCLASS >= 2
// rows).  Mixed: the FP32 cycle starts from the FP64 surface defect of every
// level, and the FP64 defect of each surface row is updated with its own
// level's matrix: b_l -= A_l c_l (UG's defect satisfies b_l = f_l - A_l x_l
// on those rows, because lmgc subtracts A_l of every correction it adds to c_l).
int NPLs::surface_iteration(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, int *err) {
  const int s = mg->lev[level].s;
  const int bl = std::min(baselevel, level);
  GMG_CHECK(xv->prec == GMG_PREC_FP64 && bv->prec == GMG_PREC_FP64,
            "ls: a locally refined hierarchy needs FP64 x and b");
  SurfLevels t;
  if (!mixed) {
    if (k_set(mg, cvec->prec, vlev(cvec, level), vlen(mg, level), 0.0)) return 1;
    if (IterNp->Iter(level, cvec, bv, Am, err)) return 1;
    surf_table(mg, bl, level, level, t);
    for (int e = 0; e < t.nlev; ++e) {
      t.mask[e] = 0;
      t.addx[e] = 1;
      t.x[e] = (double *)vlev(xv, bl + e);
      t.y[e] = vlev(cvec, bl + e);
    }
    if (k_surf_update(mg, t, cvec->prec, s)) return 1;
  } else {
    const int lo = surf_lo(mg, level);
    surf_table(mg, lo, level, level, t);
    for (int e = 0; e < t.nlev; ++e) {
      t.b[e] = (double *)vlev(bv, lo + e);
      t.b32[e] = (float *)vlev(b32, lo + e);
      t.c32[e] = lo + e == level ? (float *)vlev(cvec, level) : nullptr;
    }
    if (k_surf_prepare(mg, t, s)) return 1;
    if (IterNp->Iter(level, cvec, b32, Am, err)) return 1;
    surf_table(mg, bl, level, level, t);
    for (int e = 0; e < t.nlev; ++e) {
      t.addx[e] = 1;
      t.b[e] = (double *)vlev(bv, bl + e);
      t.x[e] = (double *)vlev(xv, bl + e);
      t.y[e] = vlev(cvec, bl + e);
    }
    if (k_surf_update(mg, t, GMG_PREC_FP32, s)) return 1;
  }
  if (surface_norm(mg, level, bv)) return 1;
  if (norm_to_host)
    GMG_CUDA(cudaMemcpyAsync(mg->norms_host, mg->norms_dev, sizeof(double) * s, cudaMemcpyDeviceToHost, mg->stream));
  return 0;
}

// the body of one ls iteration (ls.cc:694-701), enqueued without host work:
// dset(c, 0); Iter(c, b); LSUpdate x += c; norm of b into mg->norms_dev.
// Mixed: the iteration runs on FP32 copies (b32 = b; c32) and the FP64 defect
// is updated as b -= A c with the FP64 matrix (iterative refinement).
int NPLs::batch_norms(gmg_vec *bv) {
  const auto &B = mg->batch;
  if (k_batch_finish(mg, bv->prec, bv, nullptr, GMG_PREC_FP64, nullptr, false, mg->lev[0].s)) return 1;
  GMG_CUDA(cudaMemcpyAsync(B.norms_host, B.norms_dev, sizeof(double) * B.ninst * GMG_MAX_S, cudaMemcpyDeviceToHost,
                           mg->stream));
  return 0;
}

// one ls iteration of every instance of a batched hierarchy: the converged
// flags go to the device first; one lmgc cycle on the union from the deepest
// level is each instance's own cycle; then per top level x += c on the rows
// of the instances that are still iterating and their defect norms.
int NPLs::batch_iteration(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, int *err) {
  const auto &B = mg->batch;
  const int s = mg->lev[level].s;
  // on the device loop the flags stay on the device (the loop test sets them)
  if (norm_to_host) GMG_CUDA(cudaMemcpyAsync(B.conv_dev, B.conv_host, B.ninst, cudaMemcpyHostToDevice, mg->stream));
  if (!mixed) {
    // c below the deepest level is reset by every restriction of the cycle
    if (k_set(mg, cvec->prec, vlev(cvec, level), vlen(mg, level), 0.0)) return 1;
    if (IterNp->Iter(level, cvec, bv, Am, err)) return 1;
    if (k_batch_finish(mg, bv->prec, bv, xv, cvec->prec, cvec, false, s)) return 1;
  } else {
    if (k_batch_refine_prepare(mg, b32, cvec, bv)) return 1;
    // the FP32 defect the cycle leaves on the top is rebuilt from the FP64 one next time
    NPLmgc *lm = dynamic_cast<NPLmgc *>(IterNp);
    if (lm) lm->defect_unused = true;
    const int rc = IterNp->Iter(level, cvec, b32, Am, err);
    if (lm) lm->defect_unused = false;
    if (rc) return 1;
    // the FP64 refinement defect reads c in FP64: one conversion per row
    // instead of one per stored entry (conversions run on GB300's FP64 pipe)
    if (k_batch_widen(mg, c64, cvec) || k_batch_finish(mg, GMG_PREC_FP64, bv, xv, GMG_PREC_FP64, c64, true, s))
      return 1;
  }
  if (norm_to_host)
    GMG_CUDA(cudaMemcpyAsync(B.norms_host, B.norms_dev, sizeof(double) * B.ninst * GMG_MAX_S, cudaMemcpyDeviceToHost,
                             mg->stream));
  return 0;
}

int NPLs::iteration(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, int *err) {
  if (batched(level)) return batch_iteration(level, xv, bv, Am, err);
  if (mg->local()) return surface_iteration(level, xv, bv, Am, err);
  const Level &L = mg->lev[level];
  const long long len = vlen(mg, level);
  if (!mixed) {
    if (k_set(mg, cvec->prec, vlev(cvec, level), len, 0.0)) return 1;
    if (IterNp->Iter(level, cvec, bv, Am, err)) return 1;
    if (xv->prec == GMG_PREC_FP64) {
      if (k_add_mixed(mg, (double *)vlev(xv, level), cvec->prec, vlev(cvec, level), len)) return 1;
    } else if (k_add(mg, xv->prec, vlev(xv, level), vlev(cvec, level), len)) {
      return 1;
    }
  } else {
    if (k_refine_prepare(mg, (float *)vlev(b32, level), (float *)vlev(cvec, level), (const double *)vlev(bv, level),
                         len))
      return 1;
    // the FP32 defect the cycle leaves is rebuilt from the FP64 one next time
    NPLmgc *lm = dynamic_cast<NPLmgc *>(IterNp);
    if (lm) lm->defect_unused = true;
    const int rc = IterNp->Iter(level, cvec, b32, Am, err);
    if (lm) lm->defect_unused = false;
    if (rc) return 1;
    if (k_refine_update(mg, L, (double *)vlev(bv, level), (double *)vlev(xv, level), (const float *)vlev(cvec, level)))
      return 1;
  }
  if (k_nrm2x(mg, L, bv->prec, vlev(bv, level))) return 1;
  if (norm_to_host)
    GMG_CUDA(cudaMemcpyAsync(mg->norms_host, mg->norms_dev, sizeof(double) * L.s, cudaMemcpyDeviceToHost, mg->stream));
  return 0;
}

static int sc_cmp(const double *x, const double *y, int s) {  // npscan.cc:1027
  for (int i = 0; i < s; ++i)
    if (std::fabs(x[i]) >= std::fabs(y[i])) return 0;
  return 1;
}

// LinearSolver, ls.cc:637-749
int NPLs::Solver(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, const double *abs_, const double *red,
                 gmg_lresult *lr) {
  if (check_level(mg, level)) return 1;
  const int s = mg->lev[level].s;
  for (int i = 0; i < GMG_MAX_S; ++i) { reduction[i] = red[i]; abslimit[i] = abs_[i]; }
  GMG_CHECK(!mixed || (xv->prec == GMG_PREC_FP64 && bv->prec == GMG_PREC_FP64 && mg->opts.fp32_copy),
            "ls $mixed needs FP64 x and b and a hierarchy with FP32 copies");
  if (prepare_temps(bv)) return 1;
  double reach[GMG_MAX_S];
  for (int i = 0; i < s; ++i) {
    lr->first_defect[i] = lr->last_defect[i];
    reach[i] = lr->first_defect[i] * red[i];  // sc_mul_check, npscan.cc:1151
    if (reach[i] == 0.0) reach[i] = red[i];
  }
  lr->converged = sc_cmp(lr->first_defect, abs_, s);
  lr->number_of_linear_iterations = 0;
  if ((graph || loop_graph) &&
      (graph_level != level || graph_x != xv || graph_b != bv || graph_epoch != mg->graph_epoch)) {
    if (graph) cudaGraphExecDestroy(graph);
    if (loop_graph) cudaGraphExecDestroy(loop_graph);
    graph = nullptr;
    loop_graph = nullptr;
  }
  if (batched(level)) return batch_solver(level, xv, bv, Am, abs_, red, lr);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  GMG_CUDA(cudaStreamIsCapturing(mg->stream, &cap));
  const bool on_device = use_device_loop && use_graph && !loop_unavailable && IterNp->capturable() &&
                         cap == cudaStreamCaptureStatusNone;
  int i;
  for (i = 0; i < maxiter; ++i) {
    if (lr->converged) break;
    // the first iteration runs eagerly (it creates the temporaries and the
    // loop is captured after it); once the loop graph exists it runs them all
    if (on_device && (i > 0 || loop_graph)) return device_loop(i, level, xv, bv, Am, abs_, reach, lr);
    if (step(i, level, xv, bv, Am, lr) || check_iteration(i)) return 1;
    for (int r = 0; r < s; ++r) lr->last_defect[r] = mg->norms_host[r];
    for (int r = 0; r < s; ++r)
      GMG_CHECK(std::isfinite(lr->last_defect[r]), "ls: defect is not finite in iteration %d", i + 1);
    if (sc_cmp(lr->last_defect, abs_, s) || sc_cmp(lr->last_defect, reach, s)) {
      lr->converged = 1;
      lr->number_of_linear_iterations = i + 1;
      break;
    }
  }
  if (!lr->converged) lr->number_of_linear_iterations = i;
  return 0;
}

// the conditional graph of ls's loop: a WHILE node (its condition 1 at every
// launch, for the host launches it only while an iteration is due) whose body
// is one iteration, captured without the norms' copy to the host, and the
// test that counts it and sets the condition for the next pass.  Any error in
// building it leaves the host loop in charge.
int NPLs::build_loop(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am) {
  if (!loop_dev) {
    GMG_CUDA(cudaMalloc(&loop_dev, sizeof(LsLoopState)));
    GMG_CUDA(cudaMallocHost(&loop_host, sizeof(LsLoopState)));
  }
  const int ni = mg->batch.ninst;
  if (batched(level) && bloop_n != ni) {
    if (bhd_dev) cudaFree(bhd_dev);
    if (bhd_host) cudaFreeHost(bhd_host);
    if (biters_dev) cudaFree(biters_dev);
    if (blast_dev) cudaFree(blast_dev);
    if (breach_dev) cudaFree(breach_dev);
    GMG_CUDA(cudaMalloc(&bhd_dev, sizeof(BatchLoopHead)));
    GMG_CUDA(cudaMallocHost(&bhd_host, sizeof(BatchLoopHead)));
    GMG_CUDA(cudaMalloc(&biters_dev, sizeof(int) * ni));
    GMG_CUDA(cudaMalloc(&blast_dev, sizeof(double) * ni * GMG_MAX_S));
    GMG_CUDA(cudaMalloc(&breach_dev, sizeof(double) * ni * GMG_MAX_S));
    bloop_n = ni;
  }
  cudaGraph_t g = nullptr;
  GMG_CUDA(cudaGraphCreate(&g, 0));
  auto unavailable = [&](const char *what, cudaError_t e) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    loop_unavailable = true;
    if (getenv("GMG_VERBOSE")) fprintf(stderr, "ls: device loop unavailable (%s: %s)\n", what, cudaGetErrorString(e));
    return 0;
  };
  cudaGraphConditionalHandle h;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return unavailable("handle", e);
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p);
  if (e != cudaSuccess) return unavailable("conditional node", e);
  cudaGraph_t body = p.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(mg->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return unavailable("capture", e);
  const long long before = mg->launches;
  int err = 0;
  norm_to_host = false;
  int rc = iteration(level, xv, bv, Am, &err);
  norm_to_host = true;
  if (!rc)
    rc = batched(level) ? k_batch_loop_test(mg, bhd_dev, biters_dev, blast_dev, breach_dev, h)
                        : k_ls_loop_test(mg, loop_dev, iteration_flag(), h);
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(mg->stream, &captured);
  loop_kernels = mg->launches - before;
  mg->launches = before;
  // the same iteration ran eagerly before: a failure here is the capture's
  if (rc) return unavailable("capture of the iteration", cudaErrorStreamCaptureUnsupported);
  if (e != cudaSuccess) return unavailable("end capture", e);
  e = cudaGraphInstantiate(&loop_graph, g, 0);
  if (e != cudaSuccess) {
    loop_graph = nullptr;
    return unavailable("instantiate", e);
  }
  cudaGraphDestroy(g);
  graph_level = level; graph_x = xv; graph_b = bv; graph_epoch = mg->graph_epoch;
  return 0;
}

int NPLs::device_loop(int i0, int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, const double *abs_,
                      const double *reach, gmg_lresult *lr) {
  const int s = mg->lev[level].s;
  if (!loop_graph) {
    if (build_loop(level, xv, bv, Am)) return 1;
    if (!loop_graph) {  // not available on this system: the host loop from iteration i0
      int i;
      for (i = i0; i < maxiter; ++i) {
        if (step(i, level, xv, bv, Am, lr) || check_iteration(i)) return 1;
        for (int r = 0; r < s; ++r) lr->last_defect[r] = mg->norms_host[r];
        for (int r = 0; r < s; ++r)
          GMG_CHECK(std::isfinite(lr->last_defect[r]), "ls: defect is not finite in iteration %d", i + 1);
        if (sc_cmp(lr->last_defect, abs_, s) || sc_cmp(lr->last_defect, reach, s)) {
          lr->converged = 1;
          lr->number_of_linear_iterations = i + 1;
          return 0;
        }
      }
      lr->number_of_linear_iterations = i;
      return 0;
    }
  }
  LsLoopState &st = *loop_host;
  st = LsLoopState();
  st.it = i0;
  st.maxit = maxiter;
  st.s = s;
  for (int r = 0; r < s; ++r) {
    st.abs[r] = abs_[r];
    st.reach[r] = reach[r];
    st.last[r] = lr->last_defect[r];
  }
  GMG_CUDA(cudaMemcpyAsync(loop_dev, loop_host, sizeof(LsLoopState), cudaMemcpyHostToDevice, mg->stream));
  GMG_CUDA(cudaGraphLaunch(loop_graph, mg->stream));
  GMG_CUDA(cudaMemcpyAsync(loop_host, loop_dev, sizeof(LsLoopState), cudaMemcpyDeviceToHost, mg->stream));
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  mg->launches += (st.it - i0) * loop_kernels;
  if (st.flagged) {  // the solver's own error, reported as the host loop reports it
    if (fetch_iteration_flag() || check_iteration(st.flagged - 1)) return 1;
    GMG_CHECK(false, "ls: iteration flag set in iteration %d", st.flagged);
  }
  for (int r = 0; r < s; ++r) lr->last_defect[r] = st.last[r];
  GMG_CHECK(st.bad == 0, "ls: defect is not finite in iteration %d", st.bad);
  lr->converged = st.conv;
  lr->number_of_linear_iterations = st.it;
  return 0;
}

// iteration i of the solver loop, synchronised: the first runs eagerly (it
// creates the numprocs' temporaries), the following ones replay one captured
// graph of the iteration
int NPLs::step(int i, int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, gmg_lresult *lr) {
  if (step_async(i, level, xv, bv, Am, lr)) return 1;
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  return 0;
}

int NPLs::prepare_temps(gmg_vec *bv) {
  const int cprec = mixed ? GMG_PREC_FP32 : bv->prec;
  if (!cvec || cvec->prec != cprec) cvec = temp_vec(mg, name + "__c" + std::to_string(cprec), cprec);
  if (mixed && !b32) b32 = temp_vec(mg, name + "__b32", GMG_PREC_FP32);
  if (mixed && mg->batch.ninst > 0 && !c64) c64 = temp_vec(mg, name + "__c64", GMG_PREC_FP64);
  GMG_CHECK(cvec && (!mixed || b32) && (!mixed || mg->batch.ninst == 0 || c64), "ls: temporary vectors");
  return 0;
}

int NPLs::step_async(int i, int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, gmg_lresult *lr) {
  int err = 0;
  const bool graph_ok = use_graph && IterNp->capturable();
  if (graph_ok && (graph || i > 0)) {
    if (!graph) {
      cudaGraph_t g;
      const long long before = mg->launches;
      GMG_CUDA(cudaStreamBeginCapture(mg->stream, cudaStreamCaptureModeThreadLocal));
      int rc = iteration(level, xv, bv, Am, &err);
      cudaError_t ce = cudaStreamEndCapture(mg->stream, &g);
      if (rc) { if (ce == cudaSuccess) cudaGraphDestroy(g); return 1; }
      GMG_CUDA(ce);
      GMG_CUDA(cudaGraphInstantiate(&graph, g, 0));
      cudaGraphDestroy(g);
      graph_level = level; graph_x = xv; graph_b = bv; graph_epoch = mg->graph_epoch;
      graph_kernels = mg->launches - before;  // captured, not yet run
      mg->launches = before;
    }
    GMG_CUDA(cudaGraphLaunch(graph, mg->stream));
    mg->launches += graph_kernels;
  } else if (iteration(level, xv, bv, Am, &err)) {
    lr->error_code = err;
    return 1;
  }
  return 0;
}

int NPLs::batch_device_loop(int i0, int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, const double *abs_,
                            const std::vector<double> &reach, int *iters) {
  auto &B = mg->batch;
  const int s = mg->lev[level].s, ni = B.ninst;
  *iters = -1;  // not run: the caller continues on the host
  if (!loop_graph) {
    if (build_loop(level, xv, bv, Am)) return 1;
    if (!loop_graph) return 0;
  }
  BatchLoopHead &hd = *bhd_host;
  hd = BatchLoopHead();
  hd.it = i0;
  hd.maxit = maxiter;
  hd.ninst = ni;
  hd.s = s;
  hd.bad_k = ni;
  for (int r = 0; r < s; ++r) hd.abs[r] = abs_[r];
  for (int k = 0; k < ni; ++k) B.conv_host[k] = uint8_t(inst_conv[k]);
  GMG_CUDA(cudaMemcpyAsync(bhd_dev, bhd_host, sizeof(BatchLoopHead), cudaMemcpyHostToDevice, mg->stream));
  GMG_CUDA(cudaMemcpyAsync(B.conv_dev, B.conv_host, ni, cudaMemcpyHostToDevice, mg->stream));
  GMG_CUDA(cudaMemcpyAsync(biters_dev, inst_iters.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, mg->stream));
  GMG_CUDA(cudaMemcpyAsync(blast_dev, inst_last.data(), sizeof(double) * ni * GMG_MAX_S, cudaMemcpyHostToDevice,
                           mg->stream));
  GMG_CUDA(cudaMemcpyAsync(breach_dev, reach.data(), sizeof(double) * ni * GMG_MAX_S, cudaMemcpyHostToDevice,
                           mg->stream));
  GMG_CUDA(cudaStreamSynchronize(mg->stream));  // the host vectors above are pageable
  GMG_CUDA(cudaGraphLaunch(loop_graph, mg->stream));
  GMG_CUDA(cudaMemcpyAsync(bhd_host, bhd_dev, sizeof(BatchLoopHead), cudaMemcpyDeviceToHost, mg->stream));
  GMG_CUDA(cudaMemcpyAsync(B.conv_host, B.conv_dev, ni, cudaMemcpyDeviceToHost, mg->stream));
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  GMG_CUDA(cudaMemcpy(inst_iters.data(), biters_dev, sizeof(int) * ni, cudaMemcpyDeviceToHost));
  GMG_CUDA(cudaMemcpy(inst_last.data(), blast_dev, sizeof(double) * ni * GMG_MAX_S, cudaMemcpyDeviceToHost));
  mg->launches += (long long)(hd.it - i0) * loop_kernels;
  GMG_CHECK(hd.bad_k >= ni, "ls: defect of instance %d is not finite in iteration %d", hd.bad_k, hd.bad_it);
  for (int k = 0; k < ni; ++k) inst_conv[k] = B.conv_host[k];
  *iters = hd.it;
  return 0;
}

// LinearSolver on a batched hierarchy: every instance keeps its own first
// defect, reduction target and convergence test (ls.cc:680-730); converged
// instances stop updating x while the others iterate.  lr receives the
// largest first / last defect over the instances, the largest iteration
// count, and converged = all converged.
int NPLs::batch_solver(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, const double *abs_, const double *red,
                       gmg_lresult *lr) {
  auto &B = mg->batch;
  const int s = mg->lev[level].s, ni = B.ninst;
  GMG_CHECK(xv->prec == GMG_PREC_FP64, "ls on a batched hierarchy needs an FP64 x");
  GMG_CHECK((int)inst_last.size() == ni * GMG_MAX_S, "ls on a batched hierarchy: Residuum must run before Solver");
  const int min_top = *std::min_element(B.top.begin(), B.top.end());
  GMG_CHECK(baselevel <= min_top, "batched ls: base level %d above the shallowest instance's top level %d", baselevel,
            min_top);
  if (const NPLmgc *m = dynamic_cast<const NPLmgc *>(IterNp))
    GMG_CHECK(m->gamma == 1, "batched ls: lmgc with gamma %d (only V-cycles advance every instance alike)", m->gamma);
  inst_first = inst_last;
  inst_iters.assign(ni, 0);
  inst_conv.assign(ni, 0);
  std::vector<double> reach(size_t(ni) * GMG_MAX_S, 0.0);
  for (int k = 0; k < ni; ++k) {
    for (int r = 0; r < s; ++r) {
      reach[k * GMG_MAX_S + r] = inst_first[k * GMG_MAX_S + r] * red[r];
      if (reach[k * GMG_MAX_S + r] == 0.0) reach[k * GMG_MAX_S + r] = red[r];
    }
    inst_conv[k] = sc_cmp(&inst_first[k * GMG_MAX_S], abs_, s);
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  GMG_CUDA(cudaStreamIsCapturing(mg->stream, &cap));
  const bool on_device = use_device_loop && use_graph && !loop_unavailable && IterNp->capturable() &&
                         cap == cudaStreamCaptureStatusNone;
  int i;
  for (i = 0; i < maxiter; ++i) {
    bool all = true;
    for (int k = 0; k < ni; ++k) {
      B.conv_host[k] = uint8_t(inst_conv[k]);
      all = all && inst_conv[k];
    }
    if (all) break;
    if (on_device && (i > 0 || loop_graph)) {  // the rest of the loop on the device
      int run = -1;
      if (batch_device_loop(i, level, xv, bv, Am, abs_, reach, &run)) return 1;
      if (run >= 0) {
        i = run;
        break;
      }
    }
    if (step(i, level, xv, bv, Am, lr)) return 1;
    for (int k = 0; k < ni; ++k) {
      if (inst_conv[k]) continue;
      const double *d = B.norms_host + size_t(k) * GMG_MAX_S;
      for (int r = 0; r < s; ++r) {
        GMG_CHECK(std::isfinite(d[r]), "ls: defect of instance %d is not finite in iteration %d", k, i + 1);
        inst_last[k * GMG_MAX_S + r] = d[r];
      }
      if (sc_cmp(d, abs_, s) || sc_cmp(d, &reach[k * GMG_MAX_S], s)) {
        inst_conv[k] = 1;
        inst_iters[k] = i + 1;
      }
    }
  }
  lr->converged = 1;
  lr->number_of_linear_iterations = 0;
  for (int r = 0; r < s; ++r) lr->first_defect[r] = lr->last_defect[r] = 0.0;
  for (int k = 0; k < ni; ++k) {
    if (!inst_conv[k]) { inst_iters[k] = i; lr->converged = 0; }
    lr->number_of_linear_iterations = std::max(lr->number_of_linear_iterations, inst_iters[k]);
    for (int r = 0; r < s; ++r) {
      lr->first_defect[r] = std::max(lr->first_defect[r], inst_first[k * GMG_MAX_S + r]);
      lr->last_defect[r] = std::max(lr->last_defect[r], inst_last[k * GMG_MAX_S + r]);
    }
  }
  return 0;
}

int NPLs::PostProcess(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, int *result) {
  if (IterNp && IterNp->PostProcess(level, xv, bv, Am, result)) return 1;
  return 0;
}

// ------------------------------------------------------------ cg
NPCg::~NPCg() {
  if (sc) cudaFree(sc);
  if (flag_host) cudaFreeHost(flag_host);
}

int NPCg::Init(const Args &a) {  // CGInit: $r restart index (>= 0), then LinearSolverInit
  if (!a.get_int("r", &restart)) restart = 0;
  if (restart < 0) return NP_NOT_ACTIVE;
  return NPLs::Init(a);
}

std::string NPCg::Display() const {
  std::ostringstream o;
  o << NPLs::Display() << "r = " << restart << "\n";
  return o.str();
}

// CGPrepare (ls.cc:976): p = 0, rho = 1; then LinearSolver's loop
int NPCg::Solver(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, const double *abs_, const double *red,
                 gmg_lresult *lr) {
  if (check_level(mg, level)) return 1;
  GMG_CHECK(mg->batch.ninst == 0, "cg on a batched hierarchy is not supported (use ls)");
  GMG_CHECK(xv->prec == GMG_PREC_FP64 && bv->prec == GMG_PREC_FP64, "cg: x and b must be FP64");
  if (!p) p = temp_vec(mg, name + "__p", GMG_PREC_FP64);
  if (!t) t = temp_vec(mg, name + "__t", GMG_PREC_FP64);
  if (!c64) c64 = temp_vec(mg, name + "__c64", GMG_PREC_FP64);
  GMG_CHECK(p && t && c64, "cg: temporary vectors");
  if (!sc) {
    GMG_CUDA(cudaMalloc(&sc, 4 * sizeof(double)));
    GMG_CUDA(cudaMallocHost(&flag_host, sizeof(double)));
  }
  const double init[4] = {0.0, 1.0, 0.0, 0.0};
  GMG_CUDA(cudaMemcpyAsync(sc, init, sizeof init, cudaMemcpyHostToDevice, mg->stream));
  // CGPrepare, ls.cc:976: p = 0 on the levels baselevel..level
  for (int l = mg->local() ? std::min(baselevel, level) : level; l <= level; ++l)
    if (k_set(mg, GMG_PREC_FP64, vlev(p, l), vlen(mg, l), 0.0)) return 1;
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  *flag_host = 0.0;
  return NPLs::Solver(level, xv, bv, Am, abs_, red, lr);
}

// per-level tables of a Krylov iteration on a locally refined hierarchy
static SurfLevels krylov_table(gmg_mg *mg, int lo, int hi, int tl, bool all_rows, gmg_vec *bx, gmg_vec *y) {
  SurfLevels t;
  surf_table(mg, lo, hi, tl, t);
  for (int e = 0; e < t.nlev; ++e) {
    t.all[e] = all_rows;
    t.b[e] = (double *)vlev(bx, lo + e);
    t.y[e] = vlev(y, lo + e);
  }
  return t;
}

// CGUpdate (ls.cc:989-1030) on a locally refined hierarchy: every vector
// operation on the levels bl..top, with each level's matrix on all its rows;
// the dot products over UG's surface
int NPCg::surface_cg_iteration(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, int *err) {
  const int s = mg->lev[level].s, bl = std::min(baselevel, level), lo = surf_lo(mg, level);
  GMG_CHECK(lo >= bl, "cg: the surface reaches below the base level");
  gmg_vec *cv = cvec;
  if (!mixed) {
    if (k_set(mg, GMG_PREC_FP64, vlev(cvec, level), vlen(mg, level), 0.0)) return 1;
    if (IterNp->Iter(level, cvec, bv, Am, err)) return 1;
    // b += A c on every row: the defect before Iter
    if (k_surf_update(mg, krylov_table(mg, bl, level, level, true, bv, cvec), GMG_PREC_FP64, s, 1)) return 1;
  } else {
    SurfLevels t;
    surf_table(mg, lo, level, level, t);
    for (int e = 0; e < t.nlev; ++e) {
      t.b[e] = (double *)vlev(bv, lo + e);
      t.b32[e] = (float *)vlev(b32, lo + e);
      t.c32[e] = lo + e == level ? (float *)vlev(cvec, level) : nullptr;
    }
    if (k_surf_prepare(mg, t, s) || IterNp->Iter(level, cvec, b32, Am, err)) return 1;
    for (int l = bl; l <= level; ++l)
      if (k_convert(mg, GMG_PREC_FP64, vlev(c64, l), GMG_PREC_FP32, vlev(cvec, l), vlen(mg, l))) return 1;
    cv = c64;
  }
  // lambda = (c, b); p = (lambda / rho) p + c; t = -(A p); lambda = (t, p); x += alpha p; b -= alpha (A p)
  if (k_surf_dot(mg, krylov_table(mg, lo, level, level, false, cv, bv), s, 0, 1, 1.0, sc)) return 1;
  for (int l = bl; l <= level; ++l)
    if (k_cg_p(mg, vlen(mg, l), (double *)vlev(p, l), (const double *)vlev(cv, l), sc)) return 1;
  if (k_surf_update(mg, krylov_table(mg, bl, level, level, true, t, p), GMG_PREC_FP64, s, 2)) return 1;
  if (k_surf_dot(mg, krylov_table(mg, lo, level, level, false, t, p), s, 0, 2, -1.0, sc)) return 1;
  for (int l = bl; l <= level; ++l)
    if (k_cg_xb(mg, vlen(mg, l), (double *)vlev(xv, l), (const double *)vlev(p, l), (double *)vlev(bv, l),
                (const double *)vlev(t, l), sc))
      return 1;
  if (surface_norm(mg, level, bv)) return 1;
  if (norm_to_host) {
    GMG_CUDA(cudaMemcpyAsync(mg->norms_host, mg->norms_dev, sizeof(double) * s, cudaMemcpyDeviceToHost, mg->stream));
    GMG_CUDA(cudaMemcpyAsync(flag_host, sc + 3, sizeof(double), cudaMemcpyDeviceToHost, mg->stream));
  }
  return 0;
}

// one pass of LinearSolver's loop body with CGUpdate (ls.cc:694-701, 989-1064)
int NPCg::iteration(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, int *err) {
  if (mg->local()) return surface_cg_iteration(level, xv, bv, Am, err);
  const Level &L = mg->lev[level];
  const long long len = vlen(mg, level);
  double *b = (double *)vlev(bv, level), *x = (double *)vlev(xv, level), *pp = (double *)vlev(p, level),
         *tt = (double *)vlev(t, level), *c;
  if (!mixed) {
    c = (double *)vlev(cvec, level);
    if (k_set(mg, GMG_PREC_FP64, c, len, 0.0)) return 1;
    if (IterNp->Iter(level, cvec, bv, Am, err)) return 1;
    // t = A c; b += t: the defect before Iter
    if (k_set(mg, GMG_PREC_FP64, tt, len, 0.0) || k_matmul_minus(mg, L, GMG_PREC_FP64, tt, c, nullptr) ||
        k_sub(mg, len, b, tt))
      return 1;
  } else {
    // the FP32 preconditioner works on a copy of the defect
    if (k_refine_prepare(mg, (float *)vlev(b32, level), (float *)vlev(cvec, level), b, len)) return 1;
    if (IterNp->Iter(level, cvec, b32, Am, err)) return 1;
    c = (double *)vlev(c64, level);
    if (k_convert(mg, GMG_PREC_FP64, c, GMG_PREC_FP32, vlev(cvec, level), len)) return 1;
  }
  // lambda = (c, b); p = (lambda / rho) p + c; rho = lambda; t = A p;
  // lambda = (t, p); x += (rho / lambda) p; b -= (rho / lambda) t
  if (k_cg_dot(mg, L, c, b, sc, 1, 1.0) || k_cg_p(mg, len, pp, c, sc)) return 1;
  if (k_set(mg, GMG_PREC_FP64, tt, len, 0.0) || k_matmul_minus(mg, L, GMG_PREC_FP64, tt, pp, nullptr)) return 1;
  if (k_cg_dot(mg, L, tt, pp, sc, 2, -1.0) || k_cg_xb(mg, len, x, pp, b, tt, sc)) return 1;
  if (k_nrm2x(mg, L, GMG_PREC_FP64, b)) return 1;
  if (norm_to_host) {
    GMG_CUDA(cudaMemcpyAsync(mg->norms_host, mg->norms_dev, sizeof(double) * L.s, cudaMemcpyDeviceToHost, mg->stream));
    GMG_CUDA(cudaMemcpyAsync(flag_host, sc + 3, sizeof(double), cudaMemcpyDeviceToHost, mg->stream));
  }
  return 0;
}

int NPCg::fetch_iteration_flag() {
  GMG_CUDA(cudaMemcpy(flag_host, sc + 3, sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

int NPCg::check_iteration(int i) {
  GMG_CHECK(*flag_host == 0.0, "cg: (A p, p) = 0 in iteration %d", i + 1);  // CGUpdate's lambda == 0 error
  return 0;
}

// ------------------------------------------------------------ bcgs
enum { BC_RHO = 0, BC_RHONEW = 1, BC_ALPHA = 2, BC_BETA = 3, BC_OMEGA = 4, BC_TT = 5, BC_HALF = 6 };

NPBcgs::~NPBcgs() {
  if (sc) cudaFree(sc);
  if (th) cudaFree(th);
  if (half_host) cudaFreeHost(half_host);
}

int NPBcgs::Init(const Args &a) {  // BCGSInit: $R restart index (>= 0)
  if (!a.get_int("R", &restart)) restart = 0;
  if (restart < 0) return NP_NOT_ACTIVE;
  return NPLs::Init(a);
}

std::string NPBcgs::Display() const {
  std::ostringstream o;
  o << NPLs::Display() << "R = " << restart << "\n";
  return o.str();
}

// q = M^{-1} d with the preconditioner `$I`, which updates the defect it is
// given: it works on a copy (BCGSSolver saves and restores d around Iter)
int NPBcgs::precond(int level, gmg_vec *qv, gmg_vec *dv, gmg_mat *Am, int *err) {
  const long long len = vlen(mg, level);
  if (!mixed) {
    if (k_copy(mg, GMG_PREC_FP64, vlev(pc, level), vlev(dv, level), len) ||
        k_set(mg, GMG_PREC_FP64, vlev(qv, level), len, 0.0))
      return 1;
    return IterNp->Iter(level, qv, pc, Am, err);
  }
  if (k_refine_prepare(mg, (float *)vlev(b32, level), (float *)vlev(cvec, level), (const double *)vlev(dv, level), len))
    return 1;
  if (IterNp->Iter(level, cvec, b32, Am, err)) return 1;
  return k_convert(mg, GMG_PREC_FP64, vlev(qv, level), GMG_PREC_FP32, vlev(cvec, level), len);
}

// the preconditioner on every level baselevel..top of a locally refined
// hierarchy: q = lmgc(d) with d kept (Iter works on a copy / FP32 copy)
int NPBcgs::precond_levels(int level, gmg_vec *qv, gmg_vec *dv, gmg_mat *Am, int *err) {
  const int s = mg->lev[level].s, bl = std::min(baselevel, level), lo = surf_lo(mg, level);
  if (!mixed) {
    for (int l = bl; l <= level; ++l)
      if (k_copy(mg, GMG_PREC_FP64, vlev(pc, l), vlev(dv, l), vlen(mg, l))) return 1;
    if (k_set(mg, GMG_PREC_FP64, vlev(qv, level), vlen(mg, level), 0.0)) return 1;
    return IterNp->Iter(level, qv, pc, Am, err);
  }
  SurfLevels t;
  surf_table(mg, lo, level, level, t);
  for (int e = 0; e < t.nlev; ++e) {
    t.b[e] = (double *)vlev(dv, lo + e);
    t.b32[e] = (float *)vlev(b32, lo + e);
    t.c32[e] = lo + e == level ? (float *)vlev(cvec, level) : nullptr;
  }
  if (k_surf_prepare(mg, t, s) || IterNp->Iter(level, cvec, b32, Am, err)) return 1;
  for (int l = bl; l <= level; ++l)
    if (k_convert(mg, GMG_PREC_FP64, vlev(qv, l), GMG_PREC_FP32, vlev(cvec, l), vlen(mg, l))) return 1;
  return 0;
}

// BCGSSolver's loop body on a locally refined hierarchy: vector operations on
// the levels bl..top, dot products and the matrix products v = A q, t = A q
// over UG's surface (the other rows of v and t keep their values, as UG's
// dmatmul ON_SURFACE leaves them)
int NPBcgs::surface_bcgs_iteration(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, int *err) {
  const int s = mg->lev[level].s, bl = std::min(baselevel, level), lo = surf_lo(mg, level);
  GMG_CHECK(lo >= bl, "bcgs: the surface reaches below the base level");
  if (k_surf_dot(mg, krylov_table(mg, lo, level, level, false, bv, r), s, 1, 0, 1.0, sc)) return 1;
  for (int l = bl; l <= level; ++l)
    if (k_bcgs_p(mg, vlen(mg, l), (double *)vlev(p, l), (const double *)vlev(bv, l), (const double *)vlev(vn, l), sc))
      return 1;
  if (precond_levels(level, q, p, Am, err)) return 1;
  if (k_surf_update(mg, krylov_table(mg, lo, level, level, false, vn, q), GMG_PREC_FP64, s, 2)) return 1;
  if (k_surf_dot(mg, krylov_table(mg, lo, level, level, false, vn, r), s, 1, 1, -1.0, sc)) return 1;
  for (int l = bl; l <= level; ++l)
    if (k_bcgs_xs(mg, vlen(mg, l), (double *)vlev(xv, l), (const double *)vlev(q, l), (const double *)vlev(bv, l),
                  (double *)vlev(sv, l), (const double *)vlev(vn, l), sc))
      return 1;
  if (surface_norm(mg, level, sv) || k_bcgs_half_test(mg, s, th, sc)) return 1;
  GMG_CUDA(cudaMemcpyAsync(half_host, mg->norms_dev, sizeof(double) * GMG_MAX_S, cudaMemcpyDeviceToHost, mg->stream));
  GMG_CUDA(cudaMemcpyAsync(half_host + GMG_MAX_S, sc + BC_HALF, sizeof(double), cudaMemcpyDeviceToHost, mg->stream));
  if (precond_levels(level, q, sv, Am, err)) return 1;
  if (k_surf_update(mg, krylov_table(mg, lo, level, level, false, tn, q), GMG_PREC_FP64, s, 2)) return 1;
  if (k_surf_dot(mg, krylov_table(mg, lo, level, level, false, tn, tn), s, 1, 2, 1.0, sc) ||
      k_surf_dot(mg, krylov_table(mg, lo, level, level, false, sv, tn), s, 1, 3, -1.0, sc))
    return 1;
  for (int l = bl; l <= level; ++l)
    if (k_bcgs_xb(mg, vlen(mg, l), (double *)vlev(xv, l), (const double *)vlev(q, l), (double *)vlev(bv, l),
                  (const double *)vlev(sv, l), (const double *)vlev(tn, l), sc))
      return 1;
  if (surface_norm(mg, level, bv)) return 1;
  GMG_CUDA(cudaMemcpyAsync(mg->norms_host, mg->norms_dev, sizeof(double) * s, cudaMemcpyDeviceToHost, mg->stream));
  return 0;
}

// BCGSSolver's loop body (ls.cc:1904-2020) from the restart check on
int NPBcgs::iteration(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, int *err) {
  if (mg->local()) return surface_bcgs_iteration(level, xv, bv, Am, err);
  const Level &L = mg->lev[level];
  const long long len = vlen(mg, level);
  double *b = (double *)vlev(bv, level), *x = (double *)vlev(xv, level);
  double *P = (double *)vlev(p, level), *R = (double *)vlev(r, level), *V = (double *)vlev(vn, level),
         *S = (double *)vlev(sv, level), *Tn = (double *)vlev(tn, level), *Q = (double *)vlev(q, level);
  // rho_new = (b, r); beta; p = beta p + b - beta omega v
  if (k_bcgs_dot(mg, L, b, R, sc, 0, 1.0) || k_bcgs_p(mg, len, P, b, V, sc)) return 1;
  // q = M^{-1} p; v = A q (kept as -A q); alpha = rho_new / (v, r); x += alpha q; s = b - alpha v
  if (precond(level, q, p, Am, err)) return 1;
  if (k_set(mg, GMG_PREC_FP64, V, len, 0.0) || k_matmul_minus(mg, L, GMG_PREC_FP64, V, Q, nullptr)) return 1;
  if (k_bcgs_dot(mg, L, V, R, sc, 1, -1.0) || k_bcgs_xs(mg, len, x, Q, b, S, V, sc)) return 1;
  // |s| and the test after the first half step
  if (k_nrm2x(mg, L, GMG_PREC_FP64, S) || k_bcgs_half_test(mg, L.s, th, sc)) return 1;
  GMG_CUDA(cudaMemcpyAsync(half_host, mg->norms_dev, sizeof(double) * GMG_MAX_S, cudaMemcpyDeviceToHost, mg->stream));
  GMG_CUDA(cudaMemcpyAsync(half_host + GMG_MAX_S, sc + BC_HALF, sizeof(double), cudaMemcpyDeviceToHost, mg->stream));
  // q = M^{-1} s; t = A q (kept as -A q); omega = (s, t) / (t, t); x += omega q; b = s - omega t
  if (precond(level, q, sv, Am, err)) return 1;
  if (k_set(mg, GMG_PREC_FP64, Tn, len, 0.0) || k_matmul_minus(mg, L, GMG_PREC_FP64, Tn, Q, nullptr)) return 1;
  if (k_bcgs_dot(mg, L, Tn, Tn, sc, 2, 1.0) || k_bcgs_dot(mg, L, S, Tn, sc, 3, -1.0) ||
      k_bcgs_xb(mg, len, x, Q, b, S, Tn, sc))
    return 1;
  if (k_nrm2x(mg, L, GMG_PREC_FP64, b)) return 1;
  GMG_CUDA(cudaMemcpyAsync(mg->norms_host, mg->norms_dev, sizeof(double) * L.s, cudaMemcpyDeviceToHost, mg->stream));
  return 0;
}

static int sc_eq(const double *x, const double *y, double ac, int s) {  // npscan.cc:1095
  for (int i = 0; i < s; ++i)
    if (x[i] < 0.0 || y[i] < 0.0 || std::fabs(x[i] - y[i]) > ac * std::sqrt(x[i] * y[i])) return 0;
  return 1;
}

// BCGSSolver, ls.cc:1864-2062 (weights 1)
int NPBcgs::Solver(int level, gmg_vec *xv, gmg_vec *bv, gmg_mat *Am, const double *abs_, const double *red,
                   gmg_lresult *lr) {
  if (check_level(mg, level)) return 1;
  GMG_CHECK(mg->batch.ninst == 0, "bcgs on a batched hierarchy is not supported (use ls)");
  GMG_CHECK(xv->prec == GMG_PREC_FP64 && bv->prec == GMG_PREC_FP64, "bcgs: x and b must be FP64");
  GMG_CHECK(!mixed || mg->opts.fp32_copy, "bcgs $mixed needs a hierarchy with FP32 copies");
  const int s = mg->lev[level].s;
  const long long len = vlen(mg, level);
  for (int i = 0; i < GMG_MAX_S; ++i) { reduction[i] = red[i]; abslimit[i] = abs_[i]; }
  if (prepare_temps(bv)) return 1;
  gmg_vec **vs[7] = {&r, &p, &vn, &sv, &tn, &q, &pc};
  const char *nm[7] = {"__r", "__p", "__v", "__s", "__t", "__q", "__pc"};
  for (int k = 0; k < 7; ++k)
    if (!*vs[k]) {
      *vs[k] = temp_vec(mg, name + nm[k], GMG_PREC_FP64);
      GMG_CHECK(*vs[k], "bcgs: temporary vectors");
    }
  if (!sc) {
    GMG_CUDA(cudaMalloc(&sc, 8 * sizeof(double)));
    GMG_CUDA(cudaMalloc(&th, 2 * GMG_MAX_S * sizeof(double)));
    GMG_CUDA(cudaMallocHost(&half_host, (GMG_MAX_S + 1) * sizeof(double)));
  }
  double thr[2 * GMG_MAX_S] = {0}, old[GMG_MAX_S];
  for (int i = 0; i < s; ++i) {
    lr->first_defect[i] = lr->last_defect[i];
    thr[i] = abs_[i];
    thr[GMG_MAX_S + i] = lr->first_defect[i] * red[i];  // sc_mul_check, npscan.cc:1151
    if (thr[GMG_MAX_S + i] == 0.0) thr[GMG_MAX_S + i] = red[i];
    old[i] = -1.0;  // BCGSPreProcess: old_defect = -1
  }
  const double init[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};  // alpha = rho_new = beta = tt = 0
  GMG_CUDA(cudaMemcpyAsync(sc, init, sizeof init, cudaMemcpyHostToDevice, mg->stream));
  GMG_CUDA(cudaMemcpyAsync(th, thr, sizeof thr, cudaMemcpyHostToDevice, mg->stream));
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  lr->converged = sc_cmp(lr->first_defect, abs_, s);
  lr->number_of_linear_iterations = 0;
  if (graph && (graph_level != level || graph_x != xv || graph_b != bv || graph_epoch != mg->graph_epoch)) {
    cudaGraphExecDestroy(graph);
    graph = nullptr;
  }
  int eq_count = 0, its = 0;
  for (int i = 0; i < maxiter; ++i) {
    if (lr->converged) break;
    if ((restart > 0 && i % restart == 0) || i == 0) {  // p = v = 0, r = b, alpha = rho = omega = 1
      for (int l = mg->local() ? std::min(baselevel, level) : level; l <= level; ++l) {
        const long long ln = vlen(mg, l);
        if (k_set(mg, GMG_PREC_FP64, vlev(p, l), ln, 0.0) || k_set(mg, GMG_PREC_FP64, vlev(vn, l), ln, 0.0) ||
            k_copy(mg, GMG_PREC_FP64, vlev(r, l), vlev(bv, l), ln))
          return 1;
      }
      GMG_CUDA(cudaMemcpyAsync(sc + BC_ALPHA, &scal_host[0], sizeof(double), cudaMemcpyHostToDevice, mg->stream));
      GMG_CUDA(cudaMemcpyAsync(sc + BC_RHO, &scal_host[1], sizeof(double), cudaMemcpyHostToDevice, mg->stream));
      GMG_CUDA(cudaMemcpyAsync(sc + BC_OMEGA, &scal_host[2], sizeof(double), cudaMemcpyHostToDevice, mg->stream));
    }
    if (step(i, level, xv, bv, Am, lr)) return 1;
    const double *h = half_host;
    for (int k = 0; k < s; ++k)
      GMG_CHECK(std::isfinite(h[k]), "bcgs: defect is not finite in iteration %d", i + 1);
    ++its;
    if (h[GMG_MAX_S] != 0.0) {  // the first half step met the test: b = s
      for (int k = 0; k < s; ++k) lr->last_defect[k] = h[k];
      lr->converged = 1;
      break;
    }
    for (int k = 0; k < s; ++k) {
      lr->last_defect[k] = mg->norms_host[k];
      GMG_CHECK(std::isfinite(lr->last_defect[k]), "bcgs: defect is not finite in iteration %d", i + 1);
    }
    ++its;
    if (sc_cmp(lr->last_defect, abs_, s) || sc_cmp(lr->last_defect, thr + GMG_MAX_S, s)) {
      lr->converged = 1;
      break;
    }
    eq_count = sc_eq(lr->last_defect, old, 1e-4, s) ? eq_count + 1 : 0;
    for (int k = 0; k < s; ++k) old[k] = lr->last_defect[k];
    if (eq_count > 4) {
      lr->converged = 0;
      break;
    }
  }
  lr->number_of_linear_iterations = its;
  return 0;
}

// ------------------------------------------------------------ class registry (CreateClass)
static gmg_np *construct(const std::string &cls) {
  // the class name's last component selects the constructor (GetConstructor, numproc.cc:145)
  std::string c = cls.substr(cls.rfind('.') == std::string::npos ? 0 : cls.rfind('.') + 1);
  if (c == "gjac") return new NPJac;
  if (c == "ggs") return new NPGs;
  if (c == "gilu") return new NPIlu;
  if (c == "gex") return new NPEx;
  if (c == "glmgc") return new NPLmgc;
  if (c == "gtransfer") return new NPTransfer;
  if (c == "gls") return new NPLs;
  if (c == "gcg") return new NPCg;
  if (c == "gbcgs") return new NPBcgs;
  return nullptr;
}

}  // namespace gmg

using namespace gmg;

// ============================================================ C ABI
extern "C" {

int gmg_vec_create(gmg_mg *mg, const char *name, int precision, gmg_vec **out) {
  if (!mg || !name) { set_error("gmg_vec_create: bad arguments"); return 1; }
  GMG_CHECK(precision == GMG_PREC_FP64 || (precision == GMG_PREC_FP32), "bad precision %d", precision);
  GMG_CHECK(!mg->vecs.count(name), "vector %s exists", name);
  gmg_vec *v = temp_vec(mg, name, precision);
  if (!v) return 1;
  if (out) *out = v;
  return 0;
}

gmg_vec *gmg_vec_by_name(gmg_mg *mg, const char *name) {
  if (!mg || !name) return nullptr;
  auto it = mg->vecs.find(name);
  return it == mg->vecs.end() ? nullptr : it->second.get();
}

gmg_mat *gmg_mat_by_name(gmg_mg *mg, const char *name) {
  if (!mg || !name) return nullptr;
  auto it = mg->mats.find(name);
  return it == mg->mats.end() ? nullptr : it->second.get();
}

// host -> level of v, queued on mg's stream (the host buffer is consumed on return)
static int upload_async(gmg_vec *v, int level, const double *host) {
  gmg_mg *mg = v->mg;
  if (check_level(mg, level)) return 1;
  const Level &L = mg->lev[level];
  const size_t len = size_t(L.n) * L.s;
  if (stage_in(mg, host, 0, len)) return 1;
  return k_gather(mg, v->prec, vlev(v, level), (const double *)mg->stage_dev, L.perm_dev, L.n, L.s);
}

int gmg_vec_upload(gmg_vec *v, int level, const double *host) {
  if (!v || !host) { set_error("gmg_vec_upload: bad arguments"); return 1; }
  if (upload_async(v, level, host)) return 1;
  GMG_CUDA(cudaStreamSynchronize(v->mg->stream));
  return 0;
}

int gmg_vec_download(gmg_vec *v, int level, double *host) {
  if (!v || !host) { set_error("gmg_vec_download: bad arguments"); return 1; }
  gmg_mg *mg = v->mg;
  if (check_level(mg, level)) return 1;
  const Level &L = mg->lev[level];
  const size_t len = size_t(L.n) * L.s;
  if (k_scatter(mg, v->prec, (double *)mg->stage_dev, vlev(v, level), L.perm_dev, L.n, L.s)) return 1;
  return stage_out(mg, host, 0, len);
}

int gmg_vec_device_ptr(gmg_vec *v, int level, void **ptr) {
  if (!v || !ptr) { set_error("gmg_vec_device_ptr: bad arguments"); return 1; }
  if (check_level(v->mg, level)) return 1;
  *ptr = v->lev[level];
  return 0;
}

int gmg_np_create(gmg_mg *mg, const char *objname, const char *classname) {
  if (!mg || !objname || !classname) { set_error("gmg_np_create: bad arguments"); return 1; }
  gmg_np *np = construct(classname);
  GMG_CHECK(np, "no numproc class %s", classname);
  np->mg = mg;
  np->name = objname;
  np->cls = classname;
  mg->nps[objname].reset(np);
  return 0;
}

int gmg_np_init(gmg_mg *mg, const char *objname, const char *args, int *status) {
  gmg_np *np = gmg_np_by_name(mg, objname);
  GMG_CHECK(np, "no numproc %s", objname ? objname : "(null)");
  np->status = np->Init(Args(args));
  if (status) *status = np->status;
  return np->status == NP_NOT_ACTIVE ? 1 : 0;
}

int gmg_np_execute(gmg_mg *mg, const char *objname, const char *args) {
  gmg_np *np = gmg_np_by_name(mg, objname);
  GMG_CHECK(np, "no numproc %s", objname ? objname : "(null)");
  GMG_CHECK(np->status == NP_EXECUTABLE, "numproc %s is not executable", objname);
  return np->Execute(Args(args));
}

gmg_np *gmg_np_by_name(gmg_mg *mg, const char *objname) {
  if (!mg || !objname) return nullptr;
  auto it = mg->nps.find(objname);
  return it == mg->nps.end() ? nullptr : it->second.get();
}

int gmg_np_display(gmg_np *np, char *buf, int buflen) {
  if (!np || !buf || buflen <= 0) return 1;
  std::string s = np->Display();
  snprintf(buf, buflen, "%s", s.c_str());
  return 0;
}

static int check_vecs(const gmg_mg *mg, const char *fn, std::initializer_list<const gmg_vec *> vs, bool optional) {
  for (const gmg_vec *v : vs) {
    if (!v) {
      if (optional) continue;
      set_error("%s: vector missing", fn);
      return 1;
    }
    if (v->mg != mg) {
      set_error("%s: vector of another multigrid", fn);
      return 1;
    }
  }
  return 0;
}
// vectors of a numproc's multigrid, required / or left out (nullptr)
#define NP_VECS(...) \
  if (check_vecs(p->mg, __func__, {__VA_ARGS__}, false)) return 1;
#define NP_VECS_OPT(...) \
  if (check_vecs(p->mg, __func__, {__VA_ARGS__}, true)) return 1;

// the function-table entries take a numproc of their class whose init
// found its partners ($I, $S, $T; status NP_ACTIVE or NP_EXECUTABLE), as
// UG's parents only call numprocs that initialised
#define AS(T, np, k)                                                                               \
  T *p = (np && np->kind() == k) ? static_cast<T *>(np) : nullptr;                                 \
  if (!p) { set_error("%s: numproc of the wrong class", __func__); return 1; }                     \
  if (p->status < NP_ACTIVE) {                                                                     \
    set_error("%s: numproc %s is not initialised (status %d; npinit it with the objects it names " \
              "created first)", __func__, p->name.c_str(), p->status);                             \
    return 1;                                                                                      \
  }

int gmg_iter_preprocess(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *bl, int *result) {
  AS(NPIter, np, NPK_ITER);
  NP_VECS_OPT(x, b)
  int dummy;
  return p->PreProcess(level, x, b, A, bl ? bl : &dummy, result ? result : &dummy);
}
int gmg_iter_iter(gmg_np *np, int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, int *result) {
  AS(NPIter, np, NPK_ITER);
  NP_VECS(c, b)
  int dummy;
  return p->Iter(level, c, b, A, result ? result : &dummy);
}
int gmg_iter_smooth(gmg_np *np, int level, gmg_vec *t, gmg_vec *b, gmg_mat *A, gmg_vec *c, int steps,
                    int *result) {
  AS(NPIter, np, NPK_ITER);
  GMG_CHECK(t && b && c && steps >= 0, "gmg_iter_smooth: vectors missing or negative step count");
  GMG_CHECK(t->mg == p->mg && b->mg == p->mg && c->mg == p->mg, "gmg_iter_smooth: vectors of another multigrid");
  int dummy;
  return p->IterAccN(level, t, b, A, c, steps, result ? result : &dummy);
}
int gmg_iter_postprocess(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) {
  AS(NPIter, np, NPK_ITER);
  NP_VECS_OPT(x, b)
  int dummy;
  return p->PostProcess(level, x, b, A, result ? result : &dummy);
}
int gmg_transfer_preprocess(gmg_np *np, int *fl, int tl, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) {
  AS(NPTransfer, np, NPK_TRANSFER);
  NP_VECS_OPT(x, b)
  int dummy = 0, f0 = 0;
  return p->PreProcess(fl ? fl : &f0, tl, x, b, A, result ? result : &dummy);
}
int gmg_transfer_restrict_defect(gmg_np *np, int level, gmg_vec *to, gmg_vec *from, gmg_mat *A, const double *damp,
                                 int *result) {
  AS(NPTransfer, np, NPK_TRANSFER);
  NP_VECS(to, from)
  int dummy;
  return p->RestrictDefect(level, to, from, A, damp ? damp : p->damp, result ? result : &dummy);
}
int gmg_transfer_interpolate_correction(gmg_np *np, int level, gmg_vec *to, gmg_vec *from, gmg_mat *A,
                                        const double *damp, int *result) {
  AS(NPTransfer, np, NPK_TRANSFER);
  NP_VECS(to, from)
  int dummy;
  return p->InterpolateCorrection(level, to, from, A, damp ? damp : p->damp, result ? result : &dummy);
}
int gmg_transfer_interpolate_new_vectors(gmg_np *np, int fl, int tl, gmg_vec *x, int *result) {
  AS(NPTransfer, np, NPK_TRANSFER);
  NP_VECS(x)
  int dummy = 0;
  return p->InterpolateNewVectors(fl, tl, x, result ? result : &dummy);
}
int gmg_transfer_project_solution(gmg_np *np, int fl, int tl, gmg_vec *x, int *result) {
  AS(NPTransfer, np, NPK_TRANSFER);
  NP_VECS(x)
  int dummy = 0;
  return p->ProjectSolution(fl, tl, x, result ? result : &dummy);
}
int gmg_transfer_adapt_correction(gmg_np *np, int level, gmg_vec *c, gmg_vec *b, gmg_mat *A, int *result) {
  AS(NPTransfer, np, NPK_TRANSFER);
  NP_VECS_OPT(c, b)
  int dummy = 0;
  return p->AdaptCorrection(level, c, b, A, result ? result : &dummy);
}
int gmg_transfer_postprocess(gmg_np *np, int *fl, int tl, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) {
  AS(NPTransfer, np, NPK_TRANSFER);
  NP_VECS_OPT(x, b)
  int dummy = 0, f0 = 0;
  return p->PostProcess(fl ? fl : &f0, tl, x, b, A, result ? result : &dummy);
}
int gmg_ls_preprocess(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *bl, int *result) {
  AS(NPLinearSolver, np, NPK_LS);
  NP_VECS_OPT(x, b)
  int dummy = 0;
  return p->PreProcess(level, x, b, A, bl ? bl : &dummy, result ? result : &dummy);
}
int gmg_ls_defect(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) {
  AS(NPLinearSolver, np, NPK_LS);
  NP_VECS(x, b)
  int dummy;
  return p->Defect(level, x, b, A, result ? result : &dummy);
}
int gmg_ls_residuum(gmg_np *np, int fl, int tl, gmg_vec *x, gmg_vec *b, gmg_mat *A, gmg_lresult *lr) {
  AS(NPLinearSolver, np, NPK_LS);
  NP_VECS(b)
  NP_VECS_OPT(x)
  GMG_CHECK(lr, "gmg_ls_residuum: lr is NULL");
  return p->Residuum(fl, tl, x, b, A, lr);
}
int gmg_ls_solver(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, const double *abslimit,
                  const double *reduction, gmg_lresult *lr) {
  AS(NPLinearSolver, np, NPK_LS);
  NP_VECS(x, b)
  GMG_CHECK(lr, "gmg_ls_solver: lr is NULL");
  return p->Solver(level, x, b, A, abslimit ? abslimit : p->abslimit, reduction ? reduction : p->reduction, lr);
}
int gmg_ls_postprocess(gmg_np *np, int level, gmg_vec *x, gmg_vec *b, gmg_mat *A, int *result) {
  AS(NPLinearSolver, np, NPK_LS);
  NP_VECS_OPT(x, b)
  int dummy;
  return p->PostProcess(level, x, b, A, result ? result : &dummy);
}

// ------------------------------------------------ level kernels
#define MGV(mg, level)                                        \
  if (!mg) { set_error("%s: no multigrid", __func__); return 1; } \
  if (check_level(mg, level)) return 1;
// the vectors an entry works on: present and of this multigrid (a vector of
// another hierarchy has other levels and lengths)
#define VECS(...) \
  if (check_vecs(mg, __func__, {__VA_ARGS__}, false)) return 1;

int gmg_dset(gmg_mg *mg, int level, gmg_vec *x, double a) {
  MGV(mg, level);
  VECS(x)
  return k_set(mg, x->prec, vlev(x, level), vlen(mg, level), a);
}
int gmg_dcopy(gmg_mg *mg, int level, gmg_vec *x, gmg_vec *y) {
  MGV(mg, level);
  VECS(x, y)
  return k_convert(mg, x->prec, vlev(x, level), y->prec, vlev(y, level), vlen(mg, level));
}
int gmg_dadd(gmg_mg *mg, int level, gmg_vec *x, gmg_vec *y) {
  MGV(mg, level);
  VECS(x, y)
  if (x->prec == GMG_PREC_FP64) return k_add_mixed(mg, (double *)vlev(x, level), y->prec, vlev(y, level), vlen(mg, level));
  GMG_CHECK(y->prec == x->prec, "dadd: precision mismatch");
  return k_add(mg, x->prec, vlev(x, level), vlev(y, level), vlen(mg, level));
}
int gmg_dmatmul_minus(gmg_mg *mg, int level, gmg_vec *x, gmg_mat *, gmg_vec *y) {
  MGV(mg, level);
  VECS(x, y)
  if (x->prec == GMG_PREC_FP64) return k_matmul_minus_mixed(mg, mg->lev[level], (double *)vlev(x, level), y->prec, vlev(y, level));
  GMG_CHECK(y->prec == x->prec, "dmatmul_minus: precision mismatch");
  return k_matmul_minus(mg, mg->lev[level], x->prec, vlev(x, level), vlev(y, level), nullptr);
}
// dmatmul / dmatmul_add, ugblas.cc:3782 / 3889: x = A y, x += A y (FP64, every row)
static int matmul_op(gmg_mg *mg, int level, gmg_vec *x, gmg_vec *y, int op) {
  GMG_CHECK(x->prec == GMG_PREC_FP64, "dmatmul: x must be FP64");
  SurfLevels t;
  surf_table(mg, level, level, level, t);
  t.all[0] = 1;
  t.b[0] = (double *)vlev(x, level);
  t.y[0] = vlev(y, level);
  return k_surf_update(mg, t, y->prec, mg->lev[level].s, op);
}
int gmg_dmatmul(gmg_mg *mg, int level, gmg_vec *x, gmg_mat *, gmg_vec *y) {
  MGV(mg, level);
  VECS(x, y)
  return matmul_op(mg, level, x, y, 3);
}
int gmg_dmatmul_add(gmg_mg *mg, int level, gmg_vec *x, gmg_mat *, gmg_vec *y) {
  MGV(mg, level);
  VECS(x, y)
  return matmul_op(mg, level, x, y, 1);
}
// dscalx, ugblas.cc:2510: x *= a per component
int gmg_dscalx(gmg_mg *mg, int level, gmg_vec *x, const double *a) {
  MGV(mg, level);
  VECS(x)
  GMG_CHECK(a, "dscalx: no factors");
  double f[GMG_MAX_S];
  for (int r = 0; r < GMG_MAX_S; ++r) f[r] = r < mg->lev[level].s ? a[r] : 1.0;
  return k_scale(mg, x->prec, vlev(x, level), mg->lev[level].n, mg->lev[level].s, f);
}
// daxpyx, ugblas.cc:2875: x += a y per component
int gmg_daxpy(gmg_mg *mg, int level, gmg_vec *x, const double *a, gmg_vec *y) {
  MGV(mg, level);
  VECS(x, y)
  GMG_CHECK(a && x->prec == y->prec, "daxpy: no factors or precision mismatch");
  return k_axpy(mg, x->prec, vlev(x, level), vlev(y, level), mg->lev[level].n, mg->lev[level].s, a);
}
// ddot, ugblas.cc:3104: the sum over every row and component (FP64)
int gmg_ddot(gmg_mg *mg, int level, gmg_vec *x, gmg_vec *y, double *result) {
  MGV(mg, level);
  VECS(x, y)
  GMG_CHECK(result && x->prec == GMG_PREC_FP64 && y->prec == GMG_PREC_FP64, "ddot: FP64 vectors and a result");
  SurfLevels t;
  surf_table(mg, level, level, level, t);
  t.all[0] = 1;
  t.b[0] = (double *)vlev(x, level);
  t.y[0] = vlev(y, level);
  double *sc = mg->norms_dev;  // scratch: the norms' slot 0
  if (k_surf_dot(mg, t, mg->lev[level].s, 2, 0, 1.0, sc)) return 1;
  GMG_CUDA(cudaMemcpyAsync(mg->norms_host, sc, sizeof(double), cudaMemcpyDeviceToHost, mg->stream));
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  *result = mg->norms_host[0];
  return 0;
}
int gmg_dnrm2x(gmg_mg *mg, int level, gmg_vec *x, double *norms) {
  MGV(mg, level);
  VECS(x)
  if (k_nrm2x(mg, mg->lev[level], x->prec, vlev(x, level))) return 1;
  GMG_CUDA(cudaMemcpyAsync(mg->norms_host, mg->norms_dev, sizeof(double) * mg->lev[level].s, cudaMemcpyDeviceToHost, mg->stream));
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  for (int r = 0; r < mg->lev[level].s; ++r) norms[r] = mg->norms_host[r];
  return 0;
}
int gmg_l_jac(gmg_mg *mg, int level, gmg_vec *v, gmg_mat *, gmg_vec *d) {
  MGV(mg, level);
  VECS(v, d)
  static const double one[GMG_MAX_S] = {1, 1, 1, 1, 1, 1, 1, 1};
  return k_jac(mg, mg->lev[level], v->prec, vlev(v, level), vlev(d, level), one);
}
int gmg_l_lgs(gmg_mg *mg, int level, gmg_vec *v, gmg_mat *, gmg_vec *d) {
  MGV(mg, level);
  VECS(v, d)
  return k_gs(mg, mg->lev[level], v->prec, vlev(v, level), vlev(d, level));
}
int gmg_l_ilu_decomp(gmg_mg *mg, int level, gmg_mat *, const double *beta) {
  MGV(mg, level);
  NPIlu tmp;
  tmp.mg = mg;
  for (int i = 0; i < GMG_MAX_S; ++i) tmp.beta[i] = beta ? beta[i] : 0.0;
  mg->lev[level].ilu_ready = false;
  mg->coarse_images.clear();  // fused images hold copies of the factors
  int bl = 0, res = 0;
  return tmp.PreProcess(level, nullptr, nullptr, nullptr, &bl, &res);
}
int gmg_l_ilu_factors(gmg_mg *mg, int level, double *lu) {
  MGV(mg, level);
  const Level &L = mg->lev[level];
  GMG_CHECK(lu, "gmg_l_ilu_factors: no output array");
  GMG_CHECK(L.ilu_ready && L.ilu_dev.lu, "gmg_l_ilu_factors: level %d has no ILU factors", level);
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  GMG_CUDA(cudaMemcpy(lu, L.ilu_dev.lu, sizeof(double) * L.nnzb * L.s * L.s, cudaMemcpyDeviceToHost));
  return 0;
}
int gmg_l_luiter(gmg_mg *mg, int level, gmg_vec *v, gmg_mat *, gmg_vec *d) {
  MGV(mg, level);
  VECS(v, d)
  return k_luiter(mg, mg->lev[level], v->prec, vlev(v, level), vlev(d, level));
}
int gmg_standard_restrict(gmg_mg *mg, int level, gmg_vec *to, gmg_vec *from, const double *damp) {
  MGV(mg, level);
  VECS(to, from)
  GMG_CHECK(level >= 1, "no coarser grid");
  static const double one[GMG_MAX_S] = {1, 1, 1, 1, 1, 1, 1, 1};
  return k_restrict(mg, mg->lev[level], mg->lev[level - 1], to->prec, vlev(to, level - 1), vlev(from, level),
                    damp ? damp : one);
}
int gmg_standard_interpolate_correction(gmg_mg *mg, int level, gmg_vec *to, gmg_vec *from, const double *damp) {
  MGV(mg, level);
  VECS(to, from)
  GMG_CHECK(level >= 1, "no coarser grid");
  static const double one[GMG_MAX_S] = {1, 1, 1, 1, 1, 1, 1, 1};
  return k_interpolate(mg, mg->lev[level], to->prec, vlev(to, level), vlev(from, level - 1), damp ? damp : one, nullptr);
}

int gmg_restrict_by_matrix(gmg_mg *mg, int level, gmg_vec *to, gmg_vec *from, const double *damp) {
  MGV(mg, level);
  VECS(to, from)
  GMG_CHECK(level >= 1, "no coarser grid");
  GMG_CHECK(to && from && to->prec == from->prec, "RestrictByMatrix: vectors missing or of different precision");
  static const double one[GMG_MAX_S] = {1, 1, 1, 1, 1, 1, 1, 1};
  return k_restrict_imat(mg, mg->lev[level], mg->lev[level - 1], to->prec, vlev(to, level - 1), vlev(from, level),
                         damp ? damp : one);
}
int gmg_interpolate_correction_by_matrix(gmg_mg *mg, int level, gmg_vec *to, gmg_vec *from, const double *damp) {
  MGV(mg, level);
  VECS(to, from)
  GMG_CHECK(level >= 1, "no coarser grid");
  GMG_CHECK(to && from && to->prec == from->prec,
            "InterpolateCorrectionByMatrix: vectors missing or of different precision");
  static const double one[GMG_MAX_S] = {1, 1, 1, 1, 1, 1, 1, 1};
  return k_interpolate_imat(mg, mg->lev[level], to->prec, vlev(to, level), vlev(from, level - 1), damp ? damp : one,
                            nullptr);
}

int gmg_solve_host(gmg_mg *mg, const char *solver, const double *b_host, double *x_host, gmg_lresult *lr) {
  if (!mg || !solver || !b_host || !x_host || !lr) { set_error("gmg_solve_host: bad arguments"); return 1; }
  gmg_np *np = gmg_np_by_name(mg, solver);
  GMG_CHECK(np && np->kind() == NPK_LS, "no linear solver %s", solver);
  GMG_CHECK(np->status >= NP_ACTIVE, "linear solver %s is not initialised (status %d)", solver, np->status);
  NPLinearSolver *ls = static_cast<NPLinearSolver *>(np);
  NPLs *gls = dynamic_cast<NPLs *>(ls);
  GMG_CHECK(ls->x && ls->b && ls->A, "solver %s has no x, b or A", solver);
  const int top = int(mg->lev.size()) - 1;
  int bl = 0, res = 0;
  if (!(gls && gls->preprocessed) && ls->PreProcess(top, ls->x, ls->b, ls->A, &bl, &res)) return 1;
  *lr = gmg_lresult{};
  if (mg->batch.ninst > 0) {
    // packed instance vectors; x = 0 on every instance's top level
    if (gmg_vec_upload_packed(ls->b, b_host)) return 1;
    for (const auto &tl : mg->batch.tops)
      if (k_set(mg, ls->x->prec, vlev(ls->x, tl.level), vlen(mg, tl.level), 0.0)) return 1;
  } else if (mg->local()) {
    // every level: b as given, x = 0
    if (gmg_vec_upload_levels(ls->b, b_host)) return 1;
    for (int l = 0; l <= top; ++l)
      if (k_set(mg, ls->x->prec, vlev(ls->x, l), vlen(mg, l), 0.0)) return 1;
  } else {
    // queued: the solve runs on the same stream and the copy has consumed b_host
    if (upload_async(ls->b, top, b_host)) return 1;
    if (k_set(mg, ls->x->prec, vlev(ls->x, top), vlen(mg, top), 0.0)) return 1;
  }
  if (ls->Defect(top, ls->x, ls->b, ls->A, &res)) return 1;
  if (ls->Residuum(gls ? gls->baselevel : 0, top, ls->x, ls->b, ls->A, lr)) return 1;
  if (ls->Solver(top, ls->x, ls->b, ls->A, ls->abslimit, ls->reduction, lr)) return 1;
  if (mg->batch.ninst > 0) return gmg_vec_download_packed(ls->x, x_host);
  return mg->local() ? gmg_vec_download_levels(ls->x, x_host) : gmg_vec_download(ls->x, top, x_host);
}

// every level of v, levels concatenated, each in UG list order (one staged copy)
int gmg_vec_upload_levels(gmg_vec *v, const double *host) {
  if (!v || !host) { set_error("gmg_vec_upload_levels: bad arguments"); return 1; }
  gmg_mg *mg = v->mg;
  size_t len = 0;
  for (const auto &L : mg->lev) len += size_t(L.n) * L.s;
  GMG_CHECK(mg->local(), "gmg_vec_upload_levels: not a locally refined hierarchy");
  if (stage_in(mg, host, 0, len)) return 1;
  size_t off = 0;
  for (int l = 0; l < int(mg->lev.size()); ++l) {
    const Level &L = mg->lev[l];
    if (k_gather(mg, v->prec, vlev(v, l), (const double *)mg->stage_dev + off, L.perm_dev, L.n, L.s)) return 1;
    off += size_t(L.n) * L.s;
  }
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  return 0;
}

int gmg_vec_download_levels(gmg_vec *v, double *host) {
  if (!v || !host) { set_error("gmg_vec_download_levels: bad arguments"); return 1; }
  gmg_mg *mg = v->mg;
  GMG_CHECK(mg->local(), "gmg_vec_download_levels: not a locally refined hierarchy");
  size_t off = 0;
  for (int l = 0; l < int(mg->lev.size()); ++l) {
    const Level &L = mg->lev[l];
    if (k_scatter(mg, v->prec, (double *)mg->stage_dev + off, vlev(v, l), L.perm_dev, L.n, L.s)) return 1;
    off += size_t(L.n) * L.s;
  }
  return stage_out(mg, host, 0, off);
}

int gmg_mg_full_refine_level(const gmg_mg *mg) { return mg ? mg->frl : -1; }

static long long packed_len(const gmg_mg *mg) {
  return mg->batch.pack_off.empty() ? 0 : mg->batch.pack_off.back() * mg->lev[0].s;
}

int gmg_vec_upload_packed(gmg_vec *v, const double *host) {
  if (!v || !host) { set_error("gmg_vec_upload_packed: bad arguments"); return 1; }
  gmg_mg *mg = v->mg;
  GMG_CHECK(mg->batch.ninst > 0, "gmg_vec_upload_packed: not a batched hierarchy");
  const size_t len = size_t(packed_len(mg));
  if (stage_in(mg, host, 0, len)) return 1;
  for (const auto &tl : mg->batch.tops)
    if (k_pack_gather(mg, v->prec, vlev(v, tl.level), (const double *)mg->stage_dev, tl, mg->lev[0].s)) return 1;
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  return 0;
}

int gmg_vec_download_packed(gmg_vec *v, double *host) {
  if (!v || !host) { set_error("gmg_vec_download_packed: bad arguments"); return 1; }
  gmg_mg *mg = v->mg;
  GMG_CHECK(mg->batch.ninst > 0, "gmg_vec_download_packed: not a batched hierarchy");
  const size_t len = size_t(packed_len(mg));
  for (const auto &tl : mg->batch.tops)
    if (k_pack_scatter(mg, v->prec, (double *)mg->stage_dev, vlev(v, tl.level), tl, mg->lev[0].s)) return 1;
  return stage_out(mg, host, 0, len);
}

int gmg_ls_instance_result(gmg_np *np, int k, gmg_lresult *lr) {
  NPLs *ls = dynamic_cast<NPLs *>(np);
  GMG_CHECK(ls && lr, "gmg_ls_instance_result: not an ls numproc");
  const int ni = ls->mg->batch.ninst, s = ls->mg->lev[0].s;
  GMG_CHECK(k >= 0 && k < ni, "gmg_ls_instance_result: bad instance %d", k);
  GMG_CHECK((int)ls->inst_iters.size() == ni, "gmg_ls_instance_result: the solver has not run");
  *lr = gmg_lresult{};
  lr->converged = ls->inst_conv[k];
  lr->number_of_linear_iterations = ls->inst_iters[k];
  for (int r = 0; r < s; ++r) {
    lr->first_defect[r] = ls->inst_first[k * GMG_MAX_S + r];
    lr->last_defect[r] = ls->inst_last[k * GMG_MAX_S + r];
  }
  return 0;
}

}  // extern "C"
