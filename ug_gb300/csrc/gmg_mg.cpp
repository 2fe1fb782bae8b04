// Hierarchy construction: the flattened UG hierarchy (gmg_level_desc, UG
// VECTOR-list order) becomes a device-resident set of block-CSR levels in
// processing order, with the standard transfer as P (interpolation, rows =
// fine VECTORs) and R = P^T (restriction, rows = coarse VECTORs, gathered
// instead of scattered so no atomics are needed), inverse diagonal blocks,
// per-row VECTOR flags and the wavefront schedules of the triangular sweeps.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <condition_variable>
#include <mutex>
#include <queue>
#include <random>
#include <thread>
#include <tuple>

#include "gmg_internal.h"
#include "gmg_np.h"

namespace gmg {

static thread_local char g_err[1024] = "";
void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}
const char *last_error() { return g_err; }

// host copies into / out of the pinned staging buffers, split over a pool of
// worker threads kept for the process (a single thread moves ~10-20 GB/s,
// short of the host link; creating threads per call costs tens of us):
// one part per 512 KB, at most 8 parts, the caller copies part 0
namespace {
class CopyPool {
 public:
  static CopyPool &get() {
    static CopyPool pool;
    return pool;
  }
  void run(char *dst, const char *src, size_t bytes, int parts) {
    std::unique_lock<std::mutex> lk(m_);
    busy_.wait(lk, [&] { return pending_ == 0; });  // one copy at a time
    dst_ = dst; src_ = src; bytes_ = bytes; parts_ = parts;
    chunk_ = ((bytes + parts - 1) / parts + 63) & ~size_t(63);
    next_ = 1;
    pending_ = parts - 1;
    ++gen_;
    lk.unlock();
    work_.notify_all();
    std::memcpy(dst, src, std::min(chunk_, bytes));
    lk.lock();
    done_.wait(lk, [&] { return pending_ == 0; });
    busy_.notify_one();
  }
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    work_.notify_all();
    for (auto &t : th_) t.join();
  }

 private:
  CopyPool() {
    for (int t = 0; t < 7; ++t) th_.emplace_back([this] { loop(); });
  }
  void loop() {
    unsigned long long seen = 0;
    std::unique_lock<std::mutex> lk(m_);
    for (;;) {
      work_.wait(lk, [&] { return stop_ || (gen_ != seen && next_ < parts_); });
      if (stop_) return;
      const int part = next_++;
      if (next_ >= parts_) seen = gen_;
      const size_t o = chunk_ * size_t(part);
      char *d = dst_;
      const char *s = src_;
      const size_t n = o < bytes_ ? std::min(chunk_, bytes_ - o) : 0;
      lk.unlock();
      if (n) std::memcpy(d + o, s + o, n);
      lk.lock();
      if (--pending_ == 0) done_.notify_all();
    }
  }
  std::mutex m_;
  std::condition_variable work_, done_, busy_;
  std::vector<std::thread> th_;
  char *dst_ = nullptr;
  const char *src_ = nullptr;
  size_t bytes_ = 0, chunk_ = 0;
  int parts_ = 0, next_ = 0, pending_ = 0;
  unsigned long long gen_ = 0;
  bool stop_ = false;
};
}  // namespace

void par_copy(void *dst, const void *src, size_t bytes) {
  const size_t per = size_t(512) << 10;
  const int parts = int(std::min<size_t>(8, (bytes + per - 1) / per));
  if (parts <= 1) {
    std::memcpy(dst, src, bytes);
    return;
  }
  CopyPool::get().run(static_cast<char *>(dst), static_cast<const char *>(src), bytes, parts);
}

// Measured on GB300 with Grace (2.2 MB): pageable cudaMemcpyAsync 21-23 us
// each way, through the pinned buffer (host memcpy + copy) 124-153 us.
int stage_in(gmg_mg *mg, const double *host, size_t off, size_t n) {
  double *dev = (double *)mg->stage_dev + off;
  if (mg->direct_host) {
    GMG_CUDA(cudaMemcpyAsync(dev, host, n * sizeof(double), cudaMemcpyHostToDevice, mg->stream));
    return 0;
  }
  par_copy(mg->stage_host + off, host, n * sizeof(double));
  GMG_CUDA(cudaMemcpyAsync(dev, mg->stage_host + off, n * sizeof(double), cudaMemcpyHostToDevice, mg->stream));
  return 0;
}

int stage_out(gmg_mg *mg, double *host, size_t off, size_t n) {
  const double *dev = (const double *)mg->stage_dev + off;
  if (mg->direct_host) {
    GMG_CUDA(cudaMemcpyAsync(host, dev, n * sizeof(double), cudaMemcpyDeviceToHost, mg->stream));
    GMG_CUDA(cudaStreamSynchronize(mg->stream));
    return 0;
  }
  GMG_CUDA(cudaMemcpyAsync(mg->stage_host + off, dev, n * sizeof(double), cudaMemcpyDeviceToHost, mg->stream));
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  par_copy(host, mg->stage_host + off, n * sizeof(double));
  return 0;
}

int Arena::alloc(size_t bytes) {
  size = bytes;
  used = 0;
  if (bytes == 0) return 0;
  GMG_CUDA(cudaMalloc(&base, bytes));
  return 0;
}
void *Arena::take(size_t bytes) {
  size_t b = (bytes + 255) & ~size_t(255);
  if (used + b > size) return nullptr;
  void *p = base + used;
  used += b;
  return p;
}
void Arena::release() {
  if (base) cudaFree(base);
  base = nullptr;
  size = used = 0;
}

// ------------------------------------------------------------ small dense algebra
// Inverse of an s x s block by Gauss-Jordan with partial pivoting; s <= 2
// in closed form as InvertSmallBlock (np/algebra/block.cc:272).
int invert_block(int s, const double *m, double *inv) {
  if (s == 1) {
    if (m[0] == 0.0) return 1;
    inv[0] = 1.0 / m[0];
    return 0;
  }
  if (s == 2) {
    double det = m[0] * m[3] - m[1] * m[2];
    if (det == 0.0) return 1;
    double id = 1.0 / det;
    inv[0] = m[3] * id; inv[1] = -m[1] * id; inv[2] = -m[2] * id; inv[3] = m[0] * id;
    return 0;
  }
  std::vector<double> a(m, m + s * s);
  for (int i = 0; i < s * s; ++i) inv[i] = 0.0;
  for (int i = 0; i < s; ++i) inv[i * s + i] = 1.0;
  for (int c = 0; c < s; ++c) {
    int p = c;
    for (int r = c + 1; r < s; ++r) if (std::fabs(a[r * s + c]) > std::fabs(a[p * s + c])) p = r;
    if (a[p * s + c] == 0.0) return 1;
    if (p != c)
      for (int k = 0; k < s; ++k) { std::swap(a[p * s + k], a[c * s + k]); std::swap(inv[p * s + k], inv[c * s + k]); }
    double d = 1.0 / a[c * s + c];
    for (int k = 0; k < s; ++k) { a[c * s + k] *= d; inv[c * s + k] *= d; }
    for (int r = 0; r < s; ++r) {
      if (r == c) continue;
      double f = a[r * s + c];
      if (f == 0.0) continue;
      for (int k = 0; k < s; ++k) { a[r * s + k] -= f * a[c * s + k]; inv[r * s + k] -= f * inv[c * s + k]; }
    }
  }
  return 0;
}

// ------------------------------------------------------------ orderings and schedules
// Colouring of the (symmetrised) matrix graph by saturation degree (DSATUR,
// Brelaz 1979): repeatedly colour the uncoloured VECTOR with the most
// distinct colours among its neighbours (ties: larger degree, then smaller
// list position) with the smallest free colour.  Fewer colours mean fewer
// wavefronts per Gauss-Seidel sweep (4 instead of greedy's 8 on the
// Freudenthal tetrahedral meshes, 3 on the triangle meshes).
static std::vector<int> greedy_colour(int n, const std::vector<std::vector<int>> &adj, int *ncol) {
  std::vector<int> colour(n, -1);
  std::vector<std::vector<char>> seen(n);
  std::vector<int> sat(n, 0);
  using Key = std::tuple<int, int, int>;  // (saturation, degree, -index), max first
  std::priority_queue<Key> pq;
  for (int i = 0; i < n; ++i) pq.push(Key(0, int(adj[i].size()), -i));
  int nc = 0;
  while (!pq.empty()) {
    Key k = pq.top();
    pq.pop();
    int i = -std::get<2>(k);
    if (colour[i] >= 0 || std::get<0>(k) != sat[i]) continue;
    int c = 0;
    while (c < int(seen[i].size()) && seen[i][c]) ++c;
    colour[i] = c;
    nc = std::max(nc, c + 1);
    for (int j : adj[i]) {
      if (colour[j] >= 0) continue;
      if (int(seen[j].size()) <= c) seen[j].resize(c + 1, 0);
      if (!seen[j][c]) {
        seen[j][c] = 1;
        ++sat[j];
        pq.push(Key(sat[j], int(adj[j].size()), -j));
      }
    }
  }
  *ncol = nc;
  return colour;
}

// One colour less, as long as it can be found: tabu search for a proper
// colouring with k = ncol - 1 colours (Tabucol, Hertz & de Werra 1987),
// started from the current colouring with its last class moved to each
// vertex's least-conflicting colour.  A move recolours one conflicting
// vertex; the best non-tabu move (aspiration: any move to zero conflicts)
// among up to 2000 sampled conflicting vertices is taken, and its old
// colour stays tabu for 0.6 x (conflicting vertices) + 0..9 moves.
// Deterministic (fixed seed) and bounded by a budget of move evaluations
// (at most 2e8 per attempt), so a level whose colouring cannot shrink costs
// well under a second.  On the UG-refined cube this takes the 65^3 level from
// 9 to 8 colours and level 4 from 8 to 7; every colour less is one
// Gauss-Seidel wave less per sweep.  Empty classes are removed at the end.
// a lower bound of the clique number: the largest clique grown greedily
// from each of the first 4096 vertices through its sorted neighbours
static int clique_lower_bound(int n, const std::vector<std::vector<int>> &adj) {
  int best = n > 0 ? 1 : 0;
  std::vector<int> cl;
  for (int v = 0; v < std::min(n, 4096); ++v) {
    cl.assign(1, v);
    for (int u : adj[v]) {
      bool all = true;
      for (int w : cl)
        if (w != v && !std::binary_search(adj[u].begin(), adj[u].end(), w)) { all = false; break; }
      if (all) cl.push_back(u);
    }
    best = std::max(best, int(cl.size()));
  }
  return best;
}

static void reduce_colours(int n, const std::vector<std::vector<int>> &adj, std::vector<int> &colour, int *ncol) {
  if (n < 64 || *ncol <= 3) return;
  const int omega = clique_lower_bound(n, adj);
  std::mt19937 rng(20261204u);
  while (*ncol > 3 && *ncol > omega) {
    const int k = *ncol - 1;
    std::vector<int> c(colour);
    std::vector<int> gamma(size_t(n) * k, 0);  // gamma[v k + q]: neighbours of v with colour q
    for (int v = 0; v < n; ++v) {
      if (c[v] < k) continue;
      std::vector<int> cnt(k, 0);
      for (int u : adj[v])
        if (c[u] < k) cnt[c[u]]++;
      c[v] = int(std::min_element(cnt.begin(), cnt.end()) - cnt.begin());
    }
    long long conf = 0;
    for (int v = 0; v < n; ++v)
      for (int u : adj[v]) {
        gamma[size_t(v) * k + c[u]]++;
        if (u > v && c[u] == c[v]) ++conf;
      }
    std::vector<long long> tabu(size_t(n) * k, 0);
    std::vector<int> inconf, pos(n, -1);
    auto update = [&](int v) {
      const bool in = gamma[size_t(v) * k + c[v]] > 0;
      if (in && pos[v] < 0) {
        pos[v] = int(inconf.size());
        inconf.push_back(v);
      } else if (!in && pos[v] >= 0) {
        const int w = inconf.back();
        inconf[pos[v]] = w;
        pos[w] = pos[v];
        inconf.pop_back();
        pos[v] = -1;
      }
    };
    for (int v = 0; v < n; ++v) update(v);
    const long long budget = std::min<long long>(200000000LL, 400LL * n * k);
    long long evals = 0;
    for (long long it = 0; conf > 0 && evals < budget; ++it) {
      int bv = -1, bq = -1, bd = 1 << 30, ties = 0;
      const size_t m = inconf.size(), samp = std::min<size_t>(m, 2000);
      for (size_t q0 = 0; q0 < samp; ++q0) {
        const int v = m > samp ? inconf[rng() % m] : inconf[q0];
        const int cur = gamma[size_t(v) * k + c[v]];
        for (int q = 0; q < k; ++q) {
          if (q == c[v]) continue;
          const int d = gamma[size_t(v) * k + q] - cur;
          if (tabu[size_t(v) * k + q] > it && conf + d > 0) continue;
          if (d < bd) {
            bd = d; bv = v; bq = q; ties = 1;
          } else if (d == bd && rng() % unsigned(++ties) == 0) {
            bv = v; bq = q;
          }
        }
      }
      evals += (long long)samp * k;
      if (bv < 0) continue;
      const int old = c[bv];
      c[bv] = bq;
      conf += bd;
      for (int u : adj[bv]) {
        gamma[size_t(u) * k + old]--;
        gamma[size_t(u) * k + bq]++;
        update(u);
      }
      update(bv);
      tabu[size_t(bv) * k + old] = it + (long long)(0.6 * double(inconf.size())) + (long long)(rng() % 10);
    }
    if (conf > 0) break;
    colour.swap(c);
    *ncol = k;
  }
  // renumber the classes in use 0..ncol-1, in order
  std::vector<int> used(*ncol, 0), map(*ncol, -1);
  for (int v = 0; v < n; ++v) used[colour[v]] = 1;
  int nc = 0;
  for (int q = 0; q < *ncol; ++q)
    if (used[q]) map[q] = nc++;
  for (int v = 0; v < n; ++v) colour[v] = map[colour[v]];
  *ncol = nc;
}

// DSATUR, then as few colours as the tabu search finds
static std::vector<int> colour_graph(int n, const std::vector<std::vector<int>> &adj, int *ncol) {
  std::vector<int> colour = greedy_colour(n, adj, ncol);
  reduce_colours(n, adj, colour, ncol);
  return colour;
}

static std::vector<std::vector<int>> sym_adjacency(int n, const int *rowptr, const int *col);

// colour_graph of a CSR pattern, remembered for the process: hierarchies of
// one topology (the pools of a server, repeated creations) colour it once.
// Keyed by n, nnz and a 64-bit hash of the pattern; a hit is used only after
// checking that it is a proper colouring of this pattern.
static std::vector<int> colour_pattern(int n, const int *rowptr, const int *col,
                                       const std::vector<std::vector<int>> *adj, int *ncol) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, uint64_t>, std::pair<std::vector<int>, int>> cache;
  const int nnz = n > 0 ? rowptr[n] : 0;
  uint64_t h = 0x9e3779b97f4a7c15ull ^ uint64_t(n);
  auto mix = [&](uint64_t v) {
    h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
  };
  for (int i = 0; i <= n; ++i) mix(uint64_t(uint32_t(rowptr[i])));
  for (int k = 0; k < nnz; ++k) mix(uint64_t(uint32_t(col[k])));
  const auto key = std::make_tuple(n, nnz, h);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      const std::vector<int> &c = it->second.first;
      bool ok = int(c.size()) == n;
      for (int i = 0; ok && i < n; ++i)
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
          if (col[k] != i && c[col[k]] == c[i]) { ok = false; break; }
      if (ok) {
        *ncol = it->second.second;
        return c;
      }
    }
  }
  std::vector<int> c = adj ? colour_graph(n, *adj, ncol) : colour_graph(n, sym_adjacency(n, rowptr, col), ncol);
  std::lock_guard<std::mutex> lk(mu);
  if (cache.size() >= 64) cache.erase(cache.begin());
  cache[key] = {c, *ncol};
  return c;
}

static std::vector<std::vector<int>> sym_adjacency(int n, const int *rowptr, const int *col) {
  std::vector<std::vector<int>> adj(n);
  for (int i = 0; i < n; ++i)
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      int j = col[k];
      if (j == i) continue;
      adj[i].push_back(j);
      adj[j].push_back(i);
    }
  for (auto &a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  return adj;
}

// Subdomain order (GMG_ORDER_DOMAIN) for the level-scheduled triangular
// sweeps of ILU and Gauss-Seidel: the rows are grown, in breadth-first order
// of the matrix graph, into compact subdomains of at most DOMAIN_ROWS rows;
// the interior rows of every subdomain come first (subdomain by subdomain,
// breadth-first inside), then the interface rows (those with a neighbour in
// another subdomain), coloured among themselves and taken colour by colour.
// A sweep then has about (subdomain depth + interface colours) wavefronts
// whatever the level size, while the ILU(0) factors keep the quality of a
// breadth-first order inside every subdomain (a multicolour order decouples
// every row from its neighbours and weakens ILU(0) badly on systems).
constexpr int DOMAIN_ROWS = 64;

struct DomainOrder {
  std::vector<int> perm;    // processing order
  std::vector<int> region;  // subdomain of every (UG-order) row
  int nreg = 0, nint = 0;   // subdomains; interior rows (processing rows 0..nint)
  std::vector<int> cptr;    // interface colour c: processing rows cptr[c]..cptr[c+1]
};

static DomainOrder domain_order(int n, const std::vector<std::vector<int>> &adj) {
  std::vector<int> bfs, pos(n, -1);
  bfs.reserve(n);
  for (int s0 = 0; s0 < n; ++s0) {
    if (pos[s0] >= 0) continue;
    size_t head = bfs.size();
    pos[s0] = int(bfs.size());
    bfs.push_back(s0);
    while (head < bfs.size()) {
      const int i = bfs[head++];
      for (int j : adj[i])
        if (pos[j] < 0) { pos[j] = int(bfs.size()); bfs.push_back(j); }
    }
  }
  std::vector<int> region(n, -1), queue;
  int nreg = 0;
  for (int s0 : bfs) {
    if (region[s0] >= 0) continue;
    queue.assign(1, s0);
    region[s0] = nreg;
    int cnt = 1;
    for (size_t h = 0; h < queue.size() && cnt < DOMAIN_ROWS; ++h)
      for (int j : adj[queue[h]])
        if (region[j] < 0 && cnt < DOMAIN_ROWS) { region[j] = nreg; ++cnt; queue.push_back(j); }
    ++nreg;
  }
  std::vector<int> interior, iface;
  std::vector<char> is_iface(n, 0);
  for (int i : bfs) {
    bool in = true;
    for (int j : adj[i]) in &= region[j] == region[i];
    if (in) interior.push_back(i); else { iface.push_back(i); is_iface[i] = 1; }
  }
  std::stable_sort(interior.begin(), interior.end(), [&](int a, int b) { return region[a] < region[b]; });
  // colour the interface rows among themselves
  std::vector<int> local(n, -1);
  for (size_t k = 0; k < iface.size(); ++k) local[iface[k]] = int(k);
  std::vector<std::vector<int>> sub(iface.size());
  for (size_t k = 0; k < iface.size(); ++k)
    for (int j : adj[iface[k]])
      if (is_iface[j]) sub[k].push_back(local[j]);
  int nc = 0;
  std::vector<int> colour = colour_graph(int(iface.size()), sub, &nc);
  std::vector<int> ord(iface.size());
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return colour[a] < colour[b]; });
  DomainOrder D;
  D.nint = int(interior.size());
  D.perm = std::move(interior);
  for (int k : ord) D.perm.push_back(iface[k]);
  D.region = std::move(region);
  D.nreg = nreg;
  D.cptr.assign(nc + 1, 0);
  for (int c : colour) D.cptr[c + 1]++;
  for (int c = 0; c < nc; ++c) D.cptr[c + 1] += D.cptr[c];
  for (int &v : D.cptr) v += D.nint;
  return D;
}

// the interior rows of every subdomain grouped by wavefront: subdomain r's
// waves are wptr[wbeg[r]..wbeg[r+1]], wave w is rows[wptr[w]..wptr[w+1]]
static void domain_waves(int nint, const std::vector<int> &reg_of, const std::vector<int> &ptr,
                         const std::vector<int> &rows, int nreg, std::vector<int> &wbeg, std::vector<int> &wptr,
                         std::vector<int> &out) {
  std::vector<int> wave_of(nint, 0);
  for (int w = 0; w + 1 < int(ptr.size()); ++w)
    for (int k = ptr[w]; k < ptr[w + 1]; ++k)
      if (rows[k] < nint) wave_of[rows[k]] = w;
  out.resize(nint);
  std::iota(out.begin(), out.end(), 0);
  std::stable_sort(out.begin(), out.end(), [&](int a, int b) {
    return reg_of[a] != reg_of[b] ? reg_of[a] < reg_of[b] : wave_of[a] < wave_of[b];
  });
  wbeg.assign(1, 0);
  wptr.assign(1, 0);
  for (int r = 0, k = 0; r < nreg; ++r) {
    while (k < nint && reg_of[out[k]] == r) {
      const int w = wave_of[out[k]];
      while (k < nint && reg_of[out[k]] == r && wave_of[out[k]] == w) ++k;
      wptr.push_back(k);
    }
    wbeg.push_back(int(wptr.size()) - 1);
  }
}

// Level sets of the triangular dependency graph in processing order.
// forward: row i waits for its neighbours j < i; backward: for j > i.
static void wavefronts(int n, const std::vector<std::vector<int>> &adj, bool forward, std::vector<int> &ptr,
                       std::vector<int> &rows) {
  std::vector<int> w(n, 0);
  int nw = 0;
  if (forward) {
    for (int i = 0; i < n; ++i) {
      int m = -1;
      for (int j : adj[i]) if (j < i) m = std::max(m, w[j]);
      w[i] = m + 1;
      nw = std::max(nw, w[i] + 1);
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      int m = -1;
      for (int j : adj[i]) if (j > i) m = std::max(m, w[j]);
      w[i] = m + 1;
      nw = std::max(nw, w[i] + 1);
    }
  }
  ptr.assign(nw + 1, 0);
  for (int i = 0; i < n; ++i) ptr[w[i] + 1]++;
  for (int k = 0; k < nw; ++k) ptr[k + 1] += ptr[k];
  rows.assign(n, 0);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  if (forward) {
    for (int i = 0; i < n; ++i) rows[fill[w[i]]++] = i;
  } else {
    for (int i = n - 1; i >= 0; --i) rows[fill[w[i]]++] = i;
  }
}

// ------------------------------------------------------------ device uploads
template <class T>
static int upload(T *dst, const T *src, size_t n) {
  if (n) GMG_CUDA(cudaMemcpy(dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}
static std::vector<float> to_f32(const std::vector<double> &v) { return std::vector<float>(v.begin(), v.end()); }

static size_t al(size_t b) { return (b + 255) & ~size_t(255); }

// host-side build of one level (processing order), no device work
struct HostLevel {
  int n = 0, s = 1;
  std::vector<int> perm, iperm, rowptr, col;
  std::vector<double> val, dinv;
  std::vector<uint8_t> flags, skip;
  std::vector<int> lptr, lrows, uptr, urows;
  std::vector<int> prow, pcol, rrow, rcol;
  std::vector<double> pw, rw;
  bool all_active = true, all_reset = true, any_skip = false, contiguous = false;
  int ncolour = 0;
  // subdomain order: per-subdomain interior waves (forward / backward), interface colours
  int dom_nreg = 0, dom_nint = 0;
  std::vector<int> dom_region, dom_cptr, dom_fwbeg, dom_fwptr, dom_frows, dom_bwbeg, dom_bwptr, dom_brows;
  std::vector<int> sptr, scol;  // sliced ELLPACK (32-row slices)
  std::vector<double> sval;
  std::vector<uint8_t> snl;     // strictly lower entries per row (stored right after the diagonal)
  std::vector<int> spos;        // sliced-ELLPACK entry of every CSR entry
  bool ssplit = false;          // every row's lower count fits snl
};

constexpr int SELL_MIN_ROWS = 2048;  // smaller levels keep the CSR kernels

// Rows are stored as: the diagonal block, the strictly lower blocks (columns
// j < i), the strictly upper blocks, each part in the row's MATRIX-list
// order, then the padding.  A forward Gauss-Seidel wave then streams only
// entries 1..snl[i], the upper-triangle defect pass only the rest.
static void build_sell(HostLevel &H) {
  const int n = H.n, ss = H.s * H.s, ns = (n + 31) / 32;
  H.sptr.assign(ns + 1, 0);
  for (int sl = 0; sl < ns; ++sl) {
    int w = 0;
    for (int i = sl * 32; i < std::min(n, sl * 32 + 32); ++i) w = std::max(w, H.rowptr[i + 1] - H.rowptr[i]);
    H.sptr[sl + 1] = H.sptr[sl] + 32 * w;
  }
  H.scol.assign(H.sptr[ns], 0);
  H.sval.assign(size_t(H.sptr[ns]) * ss, 0.0);
  H.snl.assign(n, 0);
  H.spos.assign(H.rowptr[n], 0);
  H.ssplit = true;
  std::vector<int> order;
  for (int sl = 0; sl < ns; ++sl) {
    const int w = (H.sptr[sl + 1] - H.sptr[sl]) / 32;
    for (int lane = 0; lane < 32; ++lane) {
      const int i = sl * 32 + lane;
      order.clear();
      if (i < n) {
        const int k0 = H.rowptr[i], k1 = H.rowptr[i + 1];
        order.push_back(k0);
        for (int k = k0 + 1; k < k1; ++k)
          if (H.col[k] < i) order.push_back(k);
        const int nl = int(order.size()) - 1;
        for (int k = k0 + 1; k < k1; ++k)
          if (H.col[k] >= i) order.push_back(k);
        if (nl > 255) H.ssplit = false;
        H.snl[i] = uint8_t(std::min(nl, 255));
      }
      for (int k = 0; k < w; ++k) {
        const size_t e = size_t(H.sptr[sl]) + size_t(k) * 32 + lane;
        if (k < int(order.size())) {
          H.scol[e] = H.col[order[k]];
          H.spos[order[k]] = int(e);
          std::memcpy(&H.sval[e * ss], &H.val[size_t(order[k]) * ss], sizeof(double) * ss);
        } else {
          H.scol[e] = i < n ? i : 0;  // padding: zero block at the row itself
        }
      }
    }
  }
}

// `colour_in`, if given, is the colouring to use in GMG_ORDER_COLOR (a batched
// hierarchy passes the concatenation of its instances' own colourings)
static int build_host_level(const gmg_level_desc &d, int order, HostLevel &H,
                            const std::vector<int> *colour_in = nullptr) {
  const int n = d.n, s = d.s, ss = s * s;
  H.n = n; H.s = s;
  GMG_CHECK(n >= 0 && s >= 1 && s <= GMG_MAX_S, "bad level size n=%d s=%d", n, s);
  GMG_CHECK(n == 0 || (d.rowptr && d.col && d.val), "level arrays missing");
  for (int i = 0; i < n; ++i) {
    GMG_CHECK(d.rowptr[i + 1] > d.rowptr[i], "row %d has no diagonal entry", i);
    GMG_CHECK(d.col[d.rowptr[i]] == i, "row %d: first entry is not the diagonal (VSTART)", i);
  }
  // the symmetric adjacency is needed for a colouring or the level sets only
  std::vector<std::vector<int>> adj;
  if (!(order == GMG_ORDER_COLOR && colour_in)) adj = sym_adjacency(n, d.rowptr, d.col);
  H.perm.resize(n);
  std::iota(H.perm.begin(), H.perm.end(), 0);
  if (order == GMG_ORDER_COLOR && n > 0) {
    std::vector<int> colour;
    if (colour_in) {
      GMG_CHECK((int)colour_in->size() == n, "colouring of %zu rows for a level of %d", colour_in->size(), n);
      colour = *colour_in;
      H.ncolour = 1 + *std::max_element(colour.begin(), colour.end());
    } else {
      colour = colour_pattern(n, d.rowptr, d.col, &adj, &H.ncolour);
    }
    std::stable_sort(H.perm.begin(), H.perm.end(), [&](int a, int b) { return colour[a] < colour[b]; });
    // the wavefronts are the colour classes: contiguous ranges of the processing order
    H.lptr.assign(H.ncolour + 1, 0);
    for (int i = 0; i < n; ++i) H.lptr[colour[i] + 1]++;
    for (int c = 0; c < H.ncolour; ++c) H.lptr[c + 1] += H.lptr[c];
    H.lrows.resize(n);
    std::iota(H.lrows.begin(), H.lrows.end(), 0);
    // backward sweeps take the colours last to first
    H.uptr.assign(1, 0);
    H.urows.clear();
    for (int c = H.ncolour - 1; c >= 0; --c) {
      for (int i = H.lptr[c]; i < H.lptr[c + 1]; ++i) H.urows.push_back(i);
      H.uptr.push_back(int(H.urows.size()));
    }
    H.contiguous = true;
  } else if (order == GMG_ORDER_DOMAIN && n > 0) {
    DomainOrder D = domain_order(n, adj);
    H.perm = std::move(D.perm);
    H.dom_region = std::move(D.region);
    H.dom_nreg = D.nreg;
    H.dom_nint = D.nint;
    H.dom_cptr = std::move(D.cptr);
  }
  H.iperm.resize(n);
  for (int i = 0; i < n; ++i) H.iperm[H.perm[i]] = i;
  // matrix rows in processing order, entries in MATRIX-list order, diagonal first
  H.rowptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) H.rowptr[i + 1] = H.rowptr[i] + (d.rowptr[H.perm[i] + 1] - d.rowptr[H.perm[i]]);
  H.col.resize(H.rowptr[n]);
  H.val.resize(size_t(H.rowptr[n]) * ss);
  for (int i = 0; i < n; ++i) {
    int o = H.perm[i], k0 = d.rowptr[o], k1 = d.rowptr[o + 1], q = H.rowptr[i];
    for (int k = k0; k < k1; ++k, ++q) {
      GMG_CHECK(d.col[k] >= 0 && d.col[k] < n, "row %d: column %d out of range", o, d.col[k]);
      H.col[q] = H.iperm[d.col[k]];
      std::memcpy(&H.val[size_t(q) * ss], &d.val[size_t(k) * ss], sizeof(double) * ss);
    }
  }
  H.flags.resize(n);
  H.skip.resize(n);
  for (int i = 0; i < n; ++i) {
    int o = H.perm[i];
    int vc = d.vclass ? d.vclass[o] : 3, vn = d.vnclass ? d.vnclass[o] : 3, sk = d.skip ? d.skip[o] : 0;
    uint8_t f = 0;
    if (vc >= 3) f |= F_ACTIVE; else H.all_active = false;
    if (vc >= 2) f |= F_NEWDEF;
    if (vn >= 2) f |= F_RESET; else H.all_reset = false;
    if (vc >= 2 && vn <= 1) f |= F_FINE;
    H.flags[i] = f;
    H.skip[i] = uint8_t(sk & 0xff);
    if (sk) H.any_skip = true;
  }
  // inverse diagonal blocks (Jacobi, Gauss-Seidel)
  H.dinv.assign(size_t(n) * ss, 0.0);
  for (int i = 0; i < n; ++i) {
    if (!(H.flags[i] & F_ACTIVE)) continue;
    GMG_CHECK(!invert_block(s, &H.val[size_t(H.rowptr[i]) * ss], &H.dinv[size_t(i) * ss]),
              "singular diagonal block in row %d", H.perm[i]);
  }
  // wavefronts (level sets) of the list order
  if (!H.contiguous) {
    std::vector<std::vector<int>> padj(n);
    for (int i = 0; i < n; ++i) {
      for (int j : adj[H.perm[i]]) padj[i].push_back(H.iperm[j]);
    }
    wavefronts(n, padj, true, H.lptr, H.lrows);
    wavefronts(n, padj, false, H.uptr, H.urows);
    if (H.dom_nreg > 0) {
      std::vector<int> reg_of(H.dom_nint);
      for (int i = 0; i < H.dom_nint; ++i) reg_of[i] = H.dom_region[H.perm[i]];
      domain_waves(H.dom_nint, reg_of, H.lptr, H.lrows, H.dom_nreg, H.dom_fwbeg, H.dom_fwptr, H.dom_frows);
      domain_waves(H.dom_nint, reg_of, H.uptr, H.urows, H.dom_nreg, H.dom_bwbeg, H.dom_bwptr, H.dom_brows);
    }
  }
  if (n >= SELL_MIN_ROWS) build_sell(H);
  return 0;
}

// transfer from the coarser level `C` to `F` (processing orders of both)
static int build_host_transfer(const gmg_level_desc &d, const HostLevel &C, HostLevel &F) {
  const int n = F.n;
  GMG_CHECK(d.prowptr && d.pcol && d.pw, "transfer arrays missing on a fine level");
  F.prow.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    int o = F.perm[i];
    F.prow[i + 1] = F.prow[i] + (d.prowptr[o + 1] - d.prowptr[o]);
  }
  F.pcol.resize(F.prow[n]);
  F.pw.resize(F.prow[n]);
  for (int i = 0; i < n; ++i) {
    int o = F.perm[i], q = F.prow[i];
    for (int k = d.prowptr[o]; k < d.prowptr[o + 1]; ++k, ++q) {
      GMG_CHECK(d.pcol[k] >= 0 && d.pcol[k] < C.n, "transfer: coarse index %d out of range", d.pcol[k]);
      F.pcol[q] = C.iperm[d.pcol[k]];
      F.pw[q] = d.pw[k];
    }
  }
  // R = P^T over the fine rows with NEW_DEFECT (transgrid.cc:153)
  F.rrow.assign(C.n + 1, 0);
  for (int i = 0; i < n; ++i)
    if (F.flags[i] & F_NEWDEF)
      for (int k = F.prow[i]; k < F.prow[i + 1]; ++k) F.rrow[F.pcol[k] + 1]++;
  for (int c = 0; c < C.n; ++c) F.rrow[c + 1] += F.rrow[c];
  F.rcol.resize(F.rrow[C.n]);
  F.rw.resize(F.rrow[C.n]);
  std::vector<int> fill(F.rrow.begin(), F.rrow.end() - 1);
  for (int i = 0; i < n; ++i)
    if (F.flags[i] & F_NEWDEF)
      for (int k = F.prow[i]; k < F.prow[i + 1]; ++k) {
        int q = fill[F.pcol[k]]++;
        F.rcol[q] = i;
        F.rw[q] = F.pw[k];
      }
  return 0;
}

static int pick_tpr(const HostLevel &H) {
  if (H.n == 0) return 8;
  double avg = double(H.rowptr[H.n]) / H.n * (H.s > 1 ? 2.0 : 1.0);
  int t = avg <= 2 ? 2 : avg <= 5 ? 4 : avg <= 12 ? 8 : avg <= 24 ? 16 : 32;
  if (H.s > 1 && t > 8) t = 8;
  return t;
}

// ------------------------------------------------------------ autotuner
// Picks each level's kernel variant by timing the level's dmatmul_minus (the
// stream every smoother and transfer kernel of the level shares) in chains
// of 8 launches: on sliced-ELLPACK levels the size-based choice, the row structure
// prefetched before the launch wait, or the plain streaming loop (with an
// evict-first matrix stream where the matrix exceeds half of L2); on CSR
// levels the threads per row.
// Median of 3 timed chains after one warm-up, in the precision the V-cycle
// uses (FP32 when the hierarchy has FP32 copies).  Levels that run chained
// Gauss-Seidel steps also time two chained steps, as lmgc's pre-smoothing
// runs them, as per-wave launches, in one thread block (gs_chain_cta_ok) and
// in clusters of 2-16 blocks (gs_chain_cluster_ok); a form must be 5 %
// faster than the best before it to be taken.
static int autotune_level(gmg_mg *mg, Level &L) {
  if (L.n < 256) return 0;
  const int prec = mg->opts.fp32_copy ? GMG_PREC_FP32 : GMG_PREC_FP64;
  void *x = nullptr, *y = nullptr, *z = nullptr;
  size_t len = size_t(L.n) * L.s;
  GMG_CUDA(cudaMalloc(&x, len * sizeof(double)));
  GMG_CUDA(cudaMalloc(&y, len * sizeof(double)));
  GMG_CUDA(cudaMalloc(&z, len * sizeof(double)));
  cudaMemsetAsync(x, 0, len * sizeof(double), mg->stream);
  cudaMemsetAsync(y, 0, len * sizeof(double), mg->stream);
  cudaMemsetAsync(z, 0, len * sizeof(double), mg->stream);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // a chain of launches, as in the cycle: programmatic dependent launch lets
  // each kernel's pre-wait part overlap its predecessor, which an isolated
  // launch would not show
  constexpr int CHAIN = 8;
  auto time_op = [&](auto op) -> float {
    std::vector<float> ts;
    for (int rep = 0; rep < 4; ++rep) {
      cudaEventRecord(e0, mg->stream);
      for (int k = 0; k < CHAIN; ++k)
        if (op()) return 1e30f;
      cudaEventRecord(e1, mg->stream);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep) ts.push_back(ms / CHAIN);
    }
    std::sort(ts.begin(), ts.end());
    return ts[ts.size() / 2];
  };
  auto time_it = [&]() -> float { return time_op([&]() { return k_matmul_minus(mg, L, prec, x, y, nullptr); }); };
  std::vector<int> forms;
  for (int cw : {1, 2, 4, 8, 16})
    if (cw == 1 ? gs_chain_cta_ok(L, prec) : gs_chain_cluster_ok(L, prec, cw)) forms.push_back(cw);
  if (!forms.empty()) {
    auto chain = [&]() { return k_gs_chain(mg, L, prec, x, y, z, 2); };
    L.cta_chain = 0;
    float best = time_op(chain);
    int pick = 0;
    for (int cw : forms) {
      L.cta_chain = cw;
      const float ms = time_op(chain);
      if (ms < 0.95f * best) {
        best = ms;
        pick = cw;
      }
    }
    L.cta_chain = pick;
    if (pick > 1) gs_chain_cluster_ok(L, GMG_PREC_FP64, pick);
  }
  float best_ms = 1e30f;
  if (L.sell) {
    // the size-based default first; another variant must be 5 % faster to
    // replace it (a back-to-back launch sees a warmer L2 than the cycle,
    // where the smoothers re-read the matrix between two products); the
    // evict-first stream only where the matrix cannot stay in L2 anyway
    const long long mbytes = L.sell_nent * ((long long)L.s * L.s * (prec == GMG_PREC_FP32 ? 4 : 8) + 4);
    const bool big = mbytes > (64ll << 20);
    int cands[3][2] = {{-1, -1}, {1, 0}, {0, big ? 1 : 0}};  // (prefetch, stream)
    int bp = -1, bs = -1;
    for (int k = 0; k < 3; ++k) {
      L.prefetch = cands[k][0];
      L.stream = cands[k][1];
      const float ms = time_it();
      if (k == 0) { best_ms = ms; continue; }
      if (ms < 0.95f * best_ms) { best_ms = ms; bp = cands[k][0]; bs = cands[k][1]; }
    }
    L.prefetch = bp;
    L.stream = bs;
  } else {
    int best = L.tpr;
    const int cands[3] = {4, 8, 16};
    for (int c : cands) {
      if (L.s > 1 && c > 8) continue;
      L.tpr = c;
      const float ms = time_it();
      if (ms < best_ms) { best_ms = ms; best = c; }
    }
    L.tpr = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(x);
  cudaFree(y);
  cudaFree(z);
  GMG_CUDA(cudaGetLastError());
  return 0;
}

}  // namespace gmg

using namespace gmg;

gmg_mg::~gmg_mg() {
  nps.clear();
  if (own_stream && stream) cudaStreamDestroy(stream);
  for (auto &kv : vecs)
    for (void *p : kv.second->lev) cudaFree(p);
  for (auto &L : lev) {
    for (void *p : L.own) cudaFree(p);
    if (L.ainv) cudaFree(L.ainv);
    L.arena.release();
  }
  if (partial) cudaFree(partial);
  if (stage_dev) cudaFree(stage_dev);
  if (norms_host) cudaFreeHost(norms_host);
  if (stage_host) cudaFreeHost(stage_host);
  if (batch.conv_host) cudaFreeHost(batch.conv_host);
  if (batch.norms_host) cudaFreeHost(batch.norms_host);
}

extern "C" {

const char *gmg_last_error(void) { return gmg::last_error(); }

}  // extern "C"

// device arrays of one level in its own arena (nc = rows of level-1, or -1 on
// level 0); the host copies the factorisations need move into the Level
static int upload_level(HostLevel &h, int nc, bool f32, Level &L) {
  const int s = h.s;
  const size_t nnz = h.rowptr[h.n], ss = size_t(s) * s;
  size_t bytes = al((h.n + 1) * 4) + al(nnz * 4) + al(nnz * ss * 8) + (f32 ? al(nnz * ss * 4) : 0);
  bytes += al(h.n * ss * 8) + (f32 ? al(h.n * ss * 4) : 0) + 2 * al(h.n) + 3 * al(h.n * 4);
  bytes += al(h.lptr.size() * 4) + al(h.uptr.size() * 4);
  if (!h.sptr.empty())
    bytes += al(h.sptr.size() * 4) + al(h.scol.size() * 4) + al(h.sval.size() * 8) + (f32 ? al(h.sval.size() * 4) : 0) +
             al(h.n);
  if (nc >= 0) {
    size_t pn = h.pcol.size(), rn = h.rcol.size();
    bytes += al((h.n + 1) * 4) + al(pn * 4) + al(pn * 8) + (f32 ? al(pn * 4) : 0);
    bytes += al((size_t(nc) + 1) * 4) + al(rn * 4) + al(rn * 8) + (f32 ? al(rn * 4) : 0);
  }
  Arena &ar = L.arena;
  if (ar.alloc(bytes)) return 1;
  L.n = h.n; L.s = s; L.nnzb = nnz;
  L.all_active = h.all_active; L.all_reset = h.all_reset; L.any_skip = h.any_skip;
  L.A.nrows = h.n; L.A.nnz = nnz;
  L.A.rowptr = ar.take_n<int>(h.n + 1);
  L.A.col = ar.take_n<int>(nnz);
  L.A.v64 = ar.take_n<double>(nnz * ss);
  if (upload(L.A.rowptr, h.rowptr.data(), h.n + 1) || upload(L.A.col, h.col.data(), nnz) ||
      upload(L.A.v64, h.val.data(), nnz * ss))
    return 1;
  L.dinv64 = ar.take_n<double>(h.n * ss);
  if (upload(L.dinv64, h.dinv.data(), h.n * ss)) return 1;
  if (f32) {
    L.A.v32 = ar.take_n<float>(nnz * ss);
    L.dinv32 = ar.take_n<float>(h.n * ss);
    auto v = to_f32(h.val), dv = to_f32(h.dinv);
    if (upload(L.A.v32, v.data(), v.size()) || upload(L.dinv32, dv.data(), dv.size())) return 1;
  }
  L.flags = ar.take_n<uint8_t>(h.n);
  L.skip = ar.take_n<uint8_t>(h.n);
  L.perm_dev = ar.take_n<int>(h.n);
  L.lower.rows = ar.take_n<int>(h.n);
  L.upper.rows = ar.take_n<int>(h.n);
  L.lower.ptr = h.lptr;
  L.upper.ptr = h.uptr;
  L.lower.ptr_dev = ar.take_n<int>(h.lptr.size());
  L.upper.ptr_dev = ar.take_n<int>(h.uptr.size());
  if (upload(L.lower.ptr_dev, h.lptr.data(), h.lptr.size()) || upload(L.upper.ptr_dev, h.uptr.data(), h.uptr.size()))
    return 1;
  if (upload(L.flags, h.flags.data(), h.n) || upload(L.skip, h.skip.data(), h.n) ||
      upload(L.perm_dev, h.perm.data(), h.n) || upload(L.lower.rows, h.lrows.data(), h.n) ||
      upload(L.upper.rows, h.urows.data(), h.n))
    return 1;
  if (nc >= 0) {
    L.P.nrows = h.n; L.P.nnz = h.pcol.size();
    L.P.rowptr = ar.take_n<int>(h.n + 1);
    L.P.col = ar.take_n<int>(h.pcol.size());
    L.P.v64 = ar.take_n<double>(h.pw.size());
    L.R.nrows = nc; L.R.nnz = h.rcol.size();
    L.R.rowptr = ar.take_n<int>(nc + 1);
    L.R.col = ar.take_n<int>(h.rcol.size());
    L.R.v64 = ar.take_n<double>(h.rw.size());
    if (upload(L.P.rowptr, h.prow.data(), h.n + 1) || upload(L.P.col, h.pcol.data(), h.pcol.size()) ||
        upload(L.P.v64, h.pw.data(), h.pw.size()) || upload(L.R.rowptr, h.rrow.data(), nc + 1) ||
        upload(L.R.col, h.rcol.data(), h.rcol.size()) || upload(L.R.v64, h.rw.data(), h.rw.size()))
      return 1;
    if (f32) {
      L.P.v32 = ar.take_n<float>(h.pw.size());
      L.R.v32 = ar.take_n<float>(h.rw.size());
      auto pw = to_f32(h.pw), rw = to_f32(h.rw);
      if (upload(L.P.v32, pw.data(), pw.size()) || upload(L.R.v32, rw.data(), rw.size())) return 1;
    }
  }
  L.tpr = pick_tpr(h);
  L.waves_contiguous = h.contiguous;
  if (!h.sptr.empty()) {
    L.sell = true;
    L.sell_nent = h.sptr.back();
    L.sell_wmax = 0;
    for (size_t q = 0; q + 1 < h.sptr.size(); ++q) L.sell_wmax = std::max(L.sell_wmax, (h.sptr[q + 1] - h.sptr[q]) / 32);
    L.sell_ptr = ar.take_n<int>(h.sptr.size());
    L.sell_col = ar.take_n<int>(h.scol.size());
    L.sell_v64 = ar.take_n<double>(h.sval.size());
    if (upload(L.sell_ptr, h.sptr.data(), h.sptr.size()) || upload(L.sell_col, h.scol.data(), h.scol.size()) ||
        upload(L.sell_v64, h.sval.data(), h.sval.size()))
      return 1;
    if (f32) {
      L.sell_v32 = ar.take_n<float>(h.sval.size());
      auto sv = to_f32(h.sval);
      if (upload(L.sell_v32, sv.data(), sv.size())) return 1;
    }
    L.sell_nl = ar.take_n<uint8_t>(h.n);
    if (upload(L.sell_nl, h.snl.data(), h.n)) return 1;
    L.sell_split = h.ssplit;
    L.h_sell_pos = std::move(h.spos);
    std::vector<int>().swap(h.sptr);
    std::vector<int>().swap(h.scol);
    std::vector<double>().swap(h.sval);
  }
  GMG_CHECK(ar.used <= ar.size, "arena overflow");
  // son of every coarse row (the fine corner copy), for StandardProject
  if (nc >= 0) {
    std::vector<int> son(nc, -1);
    for (int f = 0; f < h.n; ++f)
      if (h.prow[f + 1] - h.prow[f] == 1 && h.pw[h.prow[f]] == 1.0) son[h.pcol[h.prow[f]]] = f;
    GMG_CUDA(cudaMalloc(&L.son, sizeof(int) * std::max<size_t>(son.size(), 1)));
    L.own.push_back(L.son);
    if (!son.empty()) GMG_CUDA(cudaMemcpy(L.son, son.data(), sizeof(int) * son.size(), cudaMemcpyHostToDevice));
  }
  // subdomain tables of the triangular sweeps
  if (h.dom_nreg > 0) {
    L.dom_nreg = h.dom_nreg;
    L.dom_nint = h.dom_nint;
    L.dom_cptr = h.dom_cptr;
    L.h_dom_fwbeg = h.dom_fwbeg; L.h_dom_fwptr = h.dom_fwptr; L.h_dom_frows = h.dom_frows;
    L.h_dom_bwbeg = h.dom_bwbeg; L.h_dom_bwptr = h.dom_bwptr; L.h_dom_brows = h.dom_brows;
    std::vector<int> iface(h.n - h.dom_nint);
    std::iota(iface.begin(), iface.end(), h.dom_nint);
    auto put = [&](int **dst, const std::vector<int> &src) -> int {
      GMG_CUDA(cudaMalloc(dst, sizeof(int) * std::max<size_t>(src.size(), 1)));
      L.own.push_back(*dst);
      if (!src.empty()) GMG_CUDA(cudaMemcpy(*dst, src.data(), sizeof(int) * src.size(), cudaMemcpyHostToDevice));
      return 0;
    };
    if (put(&L.dom_fwbeg, h.dom_fwbeg) || put(&L.dom_fwptr, h.dom_fwptr) || put(&L.dom_frows, h.dom_frows) ||
        put(&L.dom_bwbeg, h.dom_bwbeg) || put(&L.dom_bwptr, h.dom_bwptr) || put(&L.dom_brows, h.dom_brows) ||
        put(&L.dom_iface, iface))
      return 1;
    // the interface sweeps in one launch per direction: colours padded to
    // multiples of 8 rows (whole warps at 4 or 8 threads per row)
    const int nc = int(h.dom_cptr.size()) - 1;
    if (nc >= 2) {
      std::vector<int> fw, bw;
      auto add = [](std::vector<int> &v, int r0, int r1) {
        for (int r = r0; r < r1; ++r) v.push_back(r);
        while (v.size() % 8) v.push_back(-1);
      };
      for (int c = 0; c < nc; ++c) add(fw, h.dom_cptr[c], h.dom_cptr[c + 1]);
      for (int c = nc - 2; c >= 0; --c) add(bw, h.dom_cptr[c], h.dom_cptr[c + 1]);
      L.iface_fw_n = int(fw.size());
      L.iface_bw_n = int(bw.size());
      const size_t ni = size_t(h.n - h.dom_nint);
      if (put(&L.iface_fw_items, fw) || put(&L.iface_bw_items, bw)) return 1;
      GMG_CUDA(cudaMalloc(&L.iface_flags, sizeof(unsigned) * 2 * std::max<size_t>(ni, 1)));
      L.own.push_back(L.iface_flags);
      GMG_CUDA(cudaMemset(L.iface_flags, 0, sizeof(unsigned) * 2 * std::max<size_t>(ni, 1)));
      GMG_CUDA(cudaMalloc(&L.iface_ctr, sizeof(unsigned) * 4));
      L.own.push_back(L.iface_ctr);
      GMG_CUDA(cudaMemset(L.iface_ctr, 0, sizeof(unsigned) * 4));
      GMG_CUDA(cudaMalloc(&L.iface_err, sizeof(int)));
      L.own.push_back(L.iface_err);
      GMG_CUDA(cudaMemset(L.iface_err, 0, sizeof(int)));
      L.iface_coop = true;
    }
  }
  // keep host copies for the ILU / base factorisations and for export
  L.perm = std::move(h.perm);
  L.h_rowptr = std::move(h.rowptr);
  L.h_col = std::move(h.col);
  L.h_val = std::move(h.val);
  L.h_flags = std::move(h.flags);
  L.h_skip = std::move(h.skip);
  return 0;
}

// the device memory a Level owns (its arena, separately allocated arrays, the base inverse)
static void free_level(Level &L) {
  for (void *p : L.own) cudaFree(p);
  L.own.clear();
  if (L.ainv) cudaFree(L.ainv);
  L.ainv = nullptr;
  L.arena.release();
}

// FULLREFINELEVEL (SetSurfaceClasses, gm/algebra.cc:2905-2921) and the pinned
// / device staging buffers (the top level, or every level of a locally refined
// hierarchy, at least stage_min doubles)
static int finish_hierarchy(gmg_mg *mg, size_t stage_min) {
  const int nlevels = int(mg->lev.size()), s = mg->lev[0].s;
  mg->frl = nlevels - 1;
  for (int l = nlevels - 1; l >= 0; --l)
    for (uint8_t f : mg->lev[l].h_flags)
      if (f & F_FINE) { mg->frl = l; break; }
  GMG_CHECK(!mg->local() || nlevels <= SURF_MAX_LEVELS, "a locally refined hierarchy has at most %d levels",
            SURF_MAX_LEVELS);
  size_t top_len = std::max(size_t(mg->lev.back().n) * s, stage_min);
  if (mg->local()) {  // host vectors of a locally refined hierarchy hold every level
    size_t all = 0;
    for (const auto &L : mg->lev) all += size_t(L.n) * s;
    top_len = std::max(top_len, all);
  }
  if (top_len == 0) top_len = 1;
  if (top_len > mg->stage_len) {
    if (mg->stage_host) cudaFreeHost(mg->stage_host);
    if (mg->stage_dev) cudaFree(mg->stage_dev);
    mg->stage_host = nullptr;
    mg->stage_dev = nullptr;
    GMG_CUDA(cudaMallocHost(&mg->stage_host, sizeof(double) * top_len));
    GMG_CUDA(cudaMalloc(&mg->stage_dev, sizeof(double) * top_len));
    mg->stage_len = top_len;
  }
  return 0;
}

// the device hierarchy of `levels`; `colours` optionally fixes each level's
// colouring, `stage_min` is the least staging length (doubles) to allocate
static int create_hierarchy(const gmg_level_desc *levels, int nlevels, const gmg_mg_opts &opts,
                            const std::vector<std::vector<int>> *colours, size_t stage_min,
                            std::unique_ptr<gmg_mg> &out) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { set_error("no CUDA device"); return 1; }
  GMG_CUDA(cudaSetDevice(opts.device));
  int pma_host_tables = 0;
  GMG_CUDA(cudaDeviceGetAttribute(&pma_host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, opts.device));
  const int s = levels[0].s;
  std::vector<HostLevel> H(nlevels);
  for (int l = 0; l < nlevels; ++l) {
    GMG_CHECK(levels[l].s == s, "all levels must have the same block size");
    if (build_host_level(levels[l], opts.order, H[l], colours ? &(*colours)[l] : nullptr)) return 1;
    if (l > 0 && build_host_transfer(levels[l], H[l - 1], H[l])) return 1;
  }
  auto mg = std::make_unique<gmg_mg>();
  mg->device = opts.device;
  mg->direct_host = pma_host_tables != 0;
  mg->opts = opts;
  // a stream of its own: the legacy default stream cannot be captured into graphs
  GMG_CUDA(cudaStreamCreateWithFlags(&mg->stream, cudaStreamNonBlocking));
  mg->own_stream = true;
  mg->lev.resize(nlevels);
  for (int l = 0; l < nlevels; ++l)
    if (upload_level(H[l], l > 0 ? H[l - 1].n : -1, opts.fp32_copy != 0, mg->lev[l])) return 1;
  if (finish_hierarchy(mg.get(), stage_min)) return 1;
  // reduction scratch: per-block partial sums, the norms, and the norm kernel's ticket counter
  const size_t scratch = sizeof(double) * (REDUCE_BLOCKS * GMG_MAX_S + GMG_MAX_S + 1);
  GMG_CUDA(cudaMalloc(&mg->partial, scratch));
  GMG_CUDA(cudaMemset(mg->partial, 0, scratch));
  mg->norms_dev = mg->partial + REDUCE_BLOCKS * GMG_MAX_S;
  GMG_CUDA(cudaMallocHost(&mg->norms_host, sizeof(double) * GMG_MAX_S));
  mg->mats["MAT"] = std::make_unique<gmg_mat>();
  mg->mats["MAT"]->name = "MAT";
  mg->mats["MAT"]->mg = mg.get();
  if (opts.autotune)
    for (auto &L : mg->lev)
      if (autotune_level(mg.get(), L)) return 1;
  GMG_CUDA(cudaDeviceSynchronize());
  out = std::move(mg);
  return 0;
}

template <class T>
static int upload_owned(Level &L, T **dst, const std::vector<T> &src) {
  GMG_CUDA(cudaMalloc(dst, sizeof(T) * (src.empty() ? 1 : src.size())));
  L.own.push_back(*dst);
  if (!src.empty()) GMG_CUDA(cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
  return 0;
}

// rows of the union level that belong to instance k, in the instance's own
// list order (as processing-order indices)
static std::vector<int> instance_rows(const Level &L, int off, int n) {
  std::vector<int> iperm(L.n), r(n);
  for (int i = 0; i < L.n; ++i) iperm[L.perm[i]] = i;
  for (int j = 0; j < n; ++j) r[j] = iperm[off + j];
  return r;
}

extern "C" {

// New matrix values of one level with the structure unchanged (e.g. the next
// assembly of a time step or Newton step): `val` in the level's
// gmg_level_desc layout.  Every device copy is rewritten in place (block
// CSR FP64/FP32, sliced ELLPACK, inverse diagonal blocks, and the ILU factors
// and base-level inverse if built); the fused coarse images are dropped and
// rebuilt on their next use, and iterations captured as CUDA graphs are
// re-captured.
// an interpolation matrix for the transfer's matrix mode (UG's IMATRIX lists)
int gmg_mg_set_imatrix(gmg_mg *mg, int level, const int *rowptr, const int *col, const double *val) {
  GMG_CHECK(mg && rowptr && col && val, "gmg_mg_set_imatrix: bad arguments");
  GMG_CHECK(level >= 1 && level < int(mg->lev.size()), "gmg_mg_set_imatrix: level %d has no coarser level", level);
  GMG_CHECK(mg->batch.ninst == 0, "gmg_mg_set_imatrix: not for batched hierarchies");
  Level &F = mg->lev[level];
  const Level &C = mg->lev[level - 1];
  const int nf = F.n, nc = C.n, s = F.s, ss = s * s;
  std::vector<int> ifp(nf), icp(nc);
  for (int i = 0; i < nf; ++i) ifp[F.perm[i]] = i;
  for (int i = 0; i < nc; ++i) icp[C.perm[i]] = i;
  const int nnz = rowptr[nf];
  for (int o = 0; o < nf; ++o)
    GMG_CHECK(rowptr[o] <= rowptr[o + 1], "gmg_mg_set_imatrix: row pointers decrease at row %d", o);
  for (int k = 0; k < nnz; ++k)
    GMG_CHECK(col[k] >= 0 && col[k] < nc, "gmg_mg_set_imatrix: coarse index %d out of range", col[k]);
  // IP: fine rows in processing order, entries in their given order
  std::vector<int> pr(nf + 1, 0), pc;
  std::vector<double> pv;
  pc.reserve(nnz);
  pv.reserve(size_t(nnz) * ss);
  for (int i = 0; i < nf; ++i) {
    const int o = F.perm[i];
    for (int k = rowptr[o]; k < rowptr[o + 1]; ++k) {
      pc.push_back(icp[col[k]]);
      pv.insert(pv.end(), val + size_t(k) * ss, val + size_t(k + 1) * ss);
    }
    pr[i + 1] = int(pc.size());
  }
  // IR: coarse rows in processing order; the NEWDEF fine rows' entries in
  // fine list order (the order RestrictByMatrix accumulates them in)
  std::vector<int> rr(nc + 1, 0), rc;
  std::vector<double> rv;
  for (int o = 0; o < nf; ++o)
    if (F.h_flags[ifp[o]] & F_NEWDEF)
      for (int k = rowptr[o]; k < rowptr[o + 1]; ++k) rr[icp[col[k]] + 1]++;
  for (int w = 0; w < nc; ++w) rr[w + 1] += rr[w];
  rc.resize(rr[nc]);
  rv.resize(size_t(rr[nc]) * ss);
  std::vector<int> fill(rr.begin(), rr.end() - 1);
  for (int o = 0; o < nf; ++o)
    if (F.h_flags[ifp[o]] & F_NEWDEF)
      for (int k = rowptr[o]; k < rowptr[o + 1]; ++k) {
        const int q = fill[icp[col[k]]]++;
        rc[q] = ifp[o];
        std::copy(val + size_t(k) * ss, val + size_t(k + 1) * ss, rv.begin() + size_t(q) * ss);
      }
  auto put = [&](auto **dst, const auto &src) -> int {
    using E = typename std::remove_reference<decltype(src)>::type::value_type;
    GMG_CUDA(cudaMalloc(dst, std::max<size_t>(src.size(), 1) * sizeof(E)));
    F.own.push_back(*dst);
    if (!src.empty()) GMG_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(E), cudaMemcpyHostToDevice));
    return 0;
  };
  DevCSR P, R;
  P.nrows = nf; P.nnz = pc.size();
  R.nrows = nc; R.nnz = rc.size();
  if (put(&P.rowptr, pr) || put(&P.col, pc) || put(&P.v64, pv) || put(&R.rowptr, rr) || put(&R.col, rc) ||
      put(&R.v64, rv))
    return 1;
  if (mg->opts.fp32_copy) {
    std::vector<float> pv32(pv.begin(), pv.end()), rv32(rv.begin(), rv.end());
    if (put(&P.v32, pv32) || put(&R.v32, rv32)) return 1;
  }
  F.IP = P;
  F.IR = R;
  F.has_imat = true;
  ++mg->graph_epoch;
  return 0;
}

int gmg_mg_update_values(gmg_mg *mg, int level, const double *val) {
  if (!mg || level < 0 || level >= int(mg->lev.size()) || !val) {
    set_error("gmg_mg_update_values: bad arguments");
    return 1;
  }
  GMG_CHECK(mg->batch.ninst == 0, "gmg_mg_update_values: not for batched hierarchies (the pools rewrite slots)");
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  Level &L = mg->lev[level];
  const int n = L.n, s = L.s, ss = s * s;
  std::vector<int> iperm(n);
  for (int i = 0; i < n; ++i) iperm[L.perm[i]] = i;
  std::vector<long long> off(size_t(n) + 1, 0);  // first entry of list row o in `val`
  for (int o = 0; o < n; ++o) off[o + 1] = off[o] + (L.h_rowptr[iperm[o] + 1] - L.h_rowptr[iperm[o]]);
  for (int i = 0; i < n; ++i) {
    const long long src = off[L.perm[i]];
    for (int k = L.h_rowptr[i]; k < L.h_rowptr[i + 1]; ++k)
      std::memcpy(&L.h_val[size_t(k) * ss], &val[size_t(src + k - L.h_rowptr[i]) * ss], sizeof(double) * ss);
  }
  GMG_CUDA(cudaMemcpy(L.A.v64, L.h_val.data(), L.h_val.size() * sizeof(double), cudaMemcpyHostToDevice));
  std::vector<double> dinv(size_t(n) * ss, 0.0);
  for (int i = 0; i < n; ++i) {
    if (!(L.h_flags[i] & F_ACTIVE)) continue;
    GMG_CHECK(!invert_block(s, &L.h_val[size_t(L.h_rowptr[i]) * ss], &dinv[size_t(i) * ss]),
              "singular diagonal block in row %d", L.perm[i]);
  }
  GMG_CUDA(cudaMemcpy(L.dinv64, dinv.data(), dinv.size() * sizeof(double), cudaMemcpyHostToDevice));
  if (L.A.v32) {
    auto v = to_f32(L.h_val), dv = to_f32(dinv);
    GMG_CUDA(cudaMemcpy(L.A.v32, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice));
    GMG_CUDA(cudaMemcpy(L.dinv32, dv.data(), dv.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (L.sell) {
    HostLevel H;
    H.n = n; H.s = s;
    H.rowptr = L.h_rowptr; H.col = L.h_col; H.val = L.h_val;
    build_sell(H);
    GMG_CHECK((long long)H.sptr.back() == L.sell_nent, "gmg_mg_update_values: sliced ELLPACK layout changed");
    GMG_CUDA(cudaMemcpy(L.sell_v64, H.sval.data(), H.sval.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (L.sell_v32) {
      auto sv = to_f32(H.sval);
      GMG_CUDA(cudaMemcpy(L.sell_v32, sv.data(), sv.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
  }
  if (refresh_factors(mg, level)) return 1;
  mg->coarse_images.clear();
  ++mg->graph_epoch;
  return 0;
}

// the kernel variant of a level: threads per row (CSR levels), prefetch
// before the launch wait and evict-first stream (sliced-ELLPACK levels; -1 =
// chosen by size)
int gmg_mg_level_cta_chain(const gmg_mg *mg, int level, int *on) {
  if (!mg || !on || level < 0 || level >= int(mg->lev.size())) {
    set_error("gmg_mg_level_cta_chain: bad arguments");
    return 1;
  }
  *on = mg->lev[level].cta_chain;
  return 0;
}

int gmg_mg_set_level_cta_chain(gmg_mg *mg, int level, int on) {
  if (!mg || level < 0 || level >= int(mg->lev.size()) ||
      !(on == 0 || on == 1 || on == 2 || on == 4 || on == 8 || on == 16)) {
    set_error("gmg_mg_set_level_cta_chain: bad arguments");
    return 1;
  }
  Level &L = mg->lev[level];
  const int prec = mg->opts.fp32_copy ? GMG_PREC_FP32 : GMG_PREC_FP64;
  if (on == 1 && !gs_chain_cta_ok(L, prec)) {
    set_error("gmg_mg_set_level_cta_chain: level %d cannot run its chained steps in one thread block "
              "(needs a multicolour sliced-ELLPACK level, all rows active, at most %d colours, t and c in %lld "
              "bytes of shared memory)",
              level, CTA_CHAIN_MAXW, CTA_CHAIN_SMEM);
    return 1;
  }
  if (on > 1 && !gs_chain_cluster_ok(L, prec, on)) {
    set_error("gmg_mg_set_level_cta_chain: level %d cannot run its chained steps in one cluster of %d thread "
              "blocks (needs a multicolour sliced-ELLPACK level, all rows active, at most %d colours, t and the "
              "c slots in %lld bytes of shared memory per block, and a device that co-schedules the cluster)",
              level, on, CTA_CHAIN_MAXW, CLUSTER_CHAIN_SMEM);
    return 1;
  }
  // the FP64 cycle of a mixed hierarchy dispatches on its own fit; decide it
  // here, outside any graph capture
  if (on > 1) gs_chain_cluster_ok(L, GMG_PREC_FP64, on);
  L.cta_chain = on;
  return 0;
}

int gmg_mg_level_variant(const gmg_mg *mg, int level, int *tpr, int *prefetch, int *stream) {
  if (!mg || level < 0 || level >= int(mg->lev.size())) { set_error("gmg_mg_level_variant: bad arguments"); return 1; }
  const Level &L = mg->lev[level];
  if (tpr) *tpr = L.sell ? 0 : L.tpr;
  if (prefetch) *prefetch = L.prefetch;
  if (stream) *stream = L.stream;
  return 0;
}

// VNEW of a level's vectors (list order), kept as row flag F_VNEW
int gmg_mg_set_new_vectors(gmg_mg *mg, int level, const int *vnew) {
  if (!mg || level < 0 || level >= int(mg->lev.size()) || !vnew) {
    set_error("gmg_mg_set_new_vectors: bad arguments");
    return 1;
  }
  Level &L = mg->lev[level];
  for (int i = 0; i < L.n; ++i) {
    uint8_t &f = L.h_flags[i];
    f = uint8_t(vnew[L.perm[i]] ? (f | F_VNEW) : (f & ~F_VNEW));
  }
  if (L.n) GMG_CUDA(cudaMemcpy(L.flags, L.h_flags.data(), L.n, cudaMemcpyHostToDevice));
  return 0;
}

int gmg_mg_create(const gmg_level_desc *levels, int nlevels, const gmg_mg_opts *opts_in, gmg_mg **out) {
  if (!out || !levels || nlevels < 1) { set_error("gmg_mg_create: bad arguments"); return 1; }
  *out = nullptr;
  gmg_mg_opts opts{};
  if (opts_in) opts = *opts_in;
  std::unique_ptr<gmg_mg> mg;
  if (create_hierarchy(levels, nlevels, opts, nullptr, 0, mg)) return 1;
  *out = mg.release();
  return 0;
}

// Levels from_level.. after an adaptation: AdaptMultiGrid (gm/refine.cc)
// changes the levels from the lowest one holding a refined or coarsened
// element upward, and the flattener re-exports only those.  The levels below
// keep every device array, ILU factor and base inverse; the new levels are
// built as gmg_mg_create builds them.  Vectors keep their values on the kept
// levels and start at zero on the new ones; fused coarse images are dropped
// and captured iterations re-captured; every linear solver runs its
// PreProcess again at its next solve (new ILU factors on the new levels).
int gmg_mg_replace_levels(gmg_mg *mg, int from_level, const gmg_level_desc *levels, int count) {
  if (!mg || !levels || count < 1) { set_error("gmg_mg_replace_levels: bad arguments"); return 1; }
  GMG_CHECK(mg->batch.ninst == 0, "gmg_mg_replace_levels: not on a batched hierarchy");
  const int old_n = int(mg->lev.size());
  GMG_CHECK(from_level >= 1 && from_level <= old_n, "gmg_mg_replace_levels: first level %d not in 1..%d", from_level,
            old_n);
  const int s = mg->lev[0].s, nl = from_level + count;
  GMG_CUDA(cudaSetDevice(mg->device));
  GMG_CUDA(cudaStreamSynchronize(mg->stream));  // nothing in flight reads the old levels
  // the kept level below, as the transfer builder sees it (its row count and
  // the processing position of every list position)
  HostLevel below;
  {
    const Level &C = mg->lev[from_level - 1];
    below.n = C.n;
    below.iperm.assign(C.n, 0);
    for (int i = 0; i < C.n; ++i) below.iperm[C.perm[i]] = i;
  }
  std::vector<HostLevel> H(count);
  for (int k = 0; k < count; ++k) {
    GMG_CHECK(levels[k].s == s, "all levels must have the same block size");
    if (build_host_level(levels[k], mg->opts.order, H[k], nullptr)) return 1;
    if (build_host_transfer(levels[k], k ? H[k - 1] : below, H[k])) return 1;
  }
  {  // a locally refined result must fit the surface tables: checked before anything changes
    bool fine_below_top = false;
    for (int l = 0; l < from_level && !fine_below_top; ++l)
      for (uint8_t f : mg->lev[l].h_flags)
        if (f & F_FINE) { fine_below_top = true; break; }
    for (int k = 0; k + 1 < count && !fine_below_top; ++k)
      for (uint8_t f : H[k].flags)
        if (f & F_FINE) { fine_below_top = true; break; }
    GMG_CHECK(!fine_below_top || nl <= SURF_MAX_LEVELS, "a locally refined hierarchy has at most %d levels",
              SURF_MAX_LEVELS);
  }
  std::vector<Level> fresh(count);
  for (int k = 0; k < count; ++k)
    if (upload_level(H[k], k ? H[k - 1].n : below.n, mg->opts.fp32_copy != 0, fresh[k])) {
      for (auto &L : fresh) free_level(L);
      return 1;
    }
  for (int l = from_level; l < old_n; ++l) free_level(mg->lev[l]);
  mg->lev.resize(from_level);
  for (auto &L : fresh) mg->lev.push_back(std::move(L));
  for (auto &kv : mg->vecs) {
    gmg_vec *v = kv.second.get();
    for (int l = from_level; l < (int)v->lev.size(); ++l)
      if (v->lev[l]) cudaFree(v->lev[l]);
    v->lev.resize(nl, nullptr);
    for (int l = from_level; l < nl; ++l) {
      const size_t len = size_t(mg->lev[l].n) * s, bytes = (len ? len : 1) * (v->prec == GMG_PREC_FP64 ? 8 : 4);
      GMG_CUDA(cudaMalloc(&v->lev[l], bytes));
      GMG_CUDA(cudaMemsetAsync(v->lev[l], 0, bytes, mg->stream));
    }
  }
  mg->coarse_images.clear();
  mg->coarse_smem_cache.clear();
  ++mg->graph_epoch;
  for (auto &kv : mg->nps)
    if (NPLs *ls = dynamic_cast<NPLs *>(kv.second.get())) ls->preprocessed = false;
  if (finish_hierarchy(mg, 0)) return 1;
  if (mg->opts.autotune)
    for (int l = from_level; l < nl; ++l)
      if (autotune_level(mg, mg->lev[l])) return 1;
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  return 0;
}

// Independent instances (each a UG hierarchy with its own depth) stored
// block-diagonally: union level l holds, in instance order, level l of every
// instance that has one.  Instance k's finest level top[k] must be its surface
// (VNCLASS < 2 on every row, as on UG's top level) and its lower levels must
// be reset by the restriction (VNCLASS >= 2): then one lmgc cycle on the union
// from the deepest level is, for every instance, the cycle it runs alone.
int gmg_mg_create_batched(const gmg_level_desc *const *instances, const int *inst_nlevels, int ninst,
                          const gmg_mg_opts *opts_in, gmg_mg **out) {
  if (!out || !instances || !inst_nlevels || ninst < 1) { set_error("gmg_mg_create_batched: bad arguments"); return 1; }
  *out = nullptr;
  gmg_mg_opts opts{};
  if (opts_in) opts = *opts_in;
  int nl = 0;
  for (int k = 0; k < ninst; ++k) {
    GMG_CHECK(instances[k] && inst_nlevels[k] >= 1, "instance %d has no levels", k);
    nl = std::max(nl, inst_nlevels[k]);
  }
  const int s = instances[0][0].s;
  struct U {
    std::vector<int> rowptr{0}, col, vclass, vnclass, skip, prow{0}, pcol;
    std::vector<double> val, pw;
  };
  std::vector<U> u(nl);
  std::vector<std::vector<int>> off(nl, std::vector<int>(ninst, -1)), colours;
  if (opts.order == GMG_ORDER_COLOR) colours.resize(nl);
  std::vector<gmg_level_desc> desc(nl);
  std::map<std::tuple<const void *, const void *, int>, std::vector<int>> colour_memo;
  for (int l = 0; l < nl; ++l) {
    U &d = u[l];
    int n = 0;
    for (int k = 0; k < ninst; ++k) {
      if (inst_nlevels[k] <= l) continue;
      const gmg_level_desc &e = instances[k][l];
      const bool top = l == inst_nlevels[k] - 1;
      GMG_CHECK(e.s == s, "instance %d level %d: block size %d, expected %d", k, l, e.s, s);
      GMG_CHECK(e.n >= 0 && (e.n == 0 || (e.rowptr && e.col && e.val)), "instance %d level %d: arrays missing", k, l);
      GMG_CHECK(l == 0 || (e.prowptr && e.pcol && e.pw), "instance %d level %d: transfer arrays missing", k, l);
      off[l][k] = n;
      for (int i = 0; i < e.n; ++i) {
        GMG_CHECK(e.rowptr[i + 1] > e.rowptr[i], "instance %d level %d row %d: no diagonal entry", k, l, i);
        for (int q = e.rowptr[i]; q < e.rowptr[i + 1]; ++q) {
          GMG_CHECK(e.col[q] >= 0 && e.col[q] < e.n, "instance %d level %d row %d: column out of range", k, l, i);
          d.col.push_back(e.col[q] + n);
        }
        d.val.insert(d.val.end(), e.val + size_t(e.rowptr[i]) * s * s, e.val + size_t(e.rowptr[i + 1]) * s * s);
        d.rowptr.push_back(int(d.col.size()));
        const int vn = e.vnclass ? e.vnclass[i] : (top ? 0 : 3);
        GMG_CHECK(top ? vn < 2 : vn >= 2,
                  "instance %d level %d row %d: VNCLASS %d (a batched instance's top level is its surface)", k, l,
                  i, vn);
        d.vclass.push_back(e.vclass ? e.vclass[i] : 3);
        d.vnclass.push_back(vn);
        d.skip.push_back(e.skip ? e.skip[i] : 0);
        if (l > 0) {
          const int nc = instances[k][l - 1].n;
          for (int q = e.prowptr[i]; q < e.prowptr[i + 1]; ++q) {
            GMG_CHECK(e.pcol[q] >= 0 && e.pcol[q] < nc, "instance %d level %d: transfer index out of range", k, l);
            d.pcol.push_back(e.pcol[q] + off[l - 1][k]);
            d.pw.push_back(e.pw[q]);
          }
          d.prow.push_back(int(d.pcol.size()));
        }
      }
      if (!colours.empty()) {
        // instances sharing one level's arrays (a pool of one topology) share its colouring
        auto key = std::make_tuple((const void *)e.rowptr, (const void *)e.col, e.n);
        auto it = colour_memo.find(key);
        if (it == colour_memo.end()) {
          int nc = 0;
          it = colour_memo.emplace(key, colour_pattern(e.n, e.rowptr, e.col, nullptr, &nc)).first;
        }
        colours[l].insert(colours[l].end(), it->second.begin(), it->second.end());
      }
      n += e.n;
    }
    desc[l] = gmg_level_desc{n, s, d.rowptr.data(), d.col.data(), d.val.data(), d.vclass.data(), d.vnclass.data(),
                             d.skip.data(), l ? d.prow.data() : nullptr, l ? d.pcol.data() : nullptr,
                             l ? d.pw.data() : nullptr};
  }
  std::vector<long long> pack_off(ninst + 1, 0);
  for (int k = 0; k < ninst; ++k) pack_off[k + 1] = pack_off[k] + instances[k][inst_nlevels[k] - 1].n;
  std::unique_ptr<gmg_mg> mg;
  if (create_hierarchy(desc.data(), nl, opts, colours.empty() ? nullptr : &colours, size_t(pack_off[ninst]) * s, mg))
    return 1;
  u.clear();
  auto &B = mg->batch;
  B.ninst = ninst;
  B.list_off = off;
  B.pack_off = pack_off;
  for (int k = 0; k < ninst; ++k) {
    B.top.push_back(inst_nlevels[k] - 1);
    B.nrows_top.push_back(instances[k][inst_nlevels[k] - 1].n);
  }
  for (int l = 0; l < nl; ++l) {
    Level &L = mg->lev[l];
    // independent blocks of this level (block-diagonal base solves)
    L.blk_ptr.assign(1, 0);
    L.blk_rows.clear();
    std::vector<int> iperm(L.n);
    for (int i = 0; i < L.n; ++i) iperm[L.perm[i]] = i;
    for (int k = 0; k < ninst; ++k) {
      if (off[l][k] < 0) continue;
      const int n = instances[k][l].n;
      std::vector<int> r(n);
      for (int j = 0; j < n; ++j) r[j] = iperm[off[l][k] + j];
      std::sort(r.begin(), r.end());
      L.blk_rows.insert(L.blk_rows.end(), r.begin(), r.end());
      L.blk_ptr.push_back(int(L.blk_rows.size()));
    }
    gmg_mg::Batch::TopLevel tl;
    tl.level = l;
    std::vector<int> ptr{0}, rows, pack, chunk_k, chunk_q{0}, inst_cptr{0};
    for (int k = 0; k < ninst; ++k) {
      if (B.top[k] != l) continue;
      const int kl = int(tl.ids.size());
      tl.ids.push_back(k);
      std::vector<int> r = instance_rows(L, off[l][k], B.nrows_top[k]);
      std::vector<std::pair<int, int>> rp(r.size());
      for (int j = 0; j < B.nrows_top[k]; ++j) rp[j] = {r[j], int(pack_off[k] + j)};
      std::sort(rp.begin(), rp.end());
      for (auto &e : rp) { rows.push_back(e.first); pack.push_back(e.second); }
      for (int q = ptr.back(); q < int(rows.size()); q += BATCH_CHUNK) {
        chunk_k.push_back(kl);
        chunk_q.push_back(std::min(q + BATCH_CHUNK, int(rows.size())));
      }
      if (rows.size() == size_t(ptr.back())) {  // an instance without rows still gets its norm
        chunk_k.push_back(kl);
        chunk_q.push_back(int(rows.size()));
      }
      ptr.push_back(int(rows.size()));
      inst_cptr.push_back(int(chunk_k.size()));
    }
    if (tl.ids.empty()) continue;
    tl.ninst = int(tl.ids.size());
    tl.nrows = int(rows.size());
    tl.nchunks = int(chunk_k.size());
    tl.chunk_k = chunk_k;
    tl.chunk_q = chunk_q;
    if (upload_owned(L, &tl.ids_dev, tl.ids) || upload_owned(L, &tl.ptr_dev, ptr) || upload_owned(L, &tl.rows_dev, rows) ||
        upload_owned(L, &tl.pack_dev, pack))
      return 1;
    B.tops.push_back(std::move(tl));
  }
  GMG_CHECK((int)B.tops.size() <= GMG_MAX_TOPS, "batched hierarchy: %zu distinct instance depths (at most %d)",
            B.tops.size(), GMG_MAX_TOPS);
  {  // all top levels' chunks in one table, each instance's chunks contiguous
    std::vector<int> ctop, cid, cq0, cq1, ic0(ninst, 0), ic1(ninst, 0);
    for (size_t t = 0; t < B.tops.size(); ++t) {
      const auto &tl = B.tops[t];
      for (int h = 0; h < tl.nchunks; ++h) {
        const int id = tl.ids[tl.chunk_k[h]];
        if (h == 0 || tl.chunk_k[h] != tl.chunk_k[h - 1]) ic0[id] = int(ctop.size());
        ctop.push_back(int(t));
        cid.push_back(id);
        cq0.push_back(tl.chunk_q[h]);
        cq1.push_back(tl.chunk_q[h + 1]);
        ic1[id] = int(ctop.size());
      }
    }
    B.nchunks_all = int(ctop.size());
    Level &T0 = mg->lev.back();
    if (upload_owned(T0, &B.chunk_top_dev, ctop) || upload_owned(T0, &B.chunk_id_dev, cid) ||
        upload_owned(T0, &B.chunk_q0_dev, cq0) || upload_owned(T0, &B.chunk_q1_dev, cq1) ||
        upload_owned(T0, &B.inst_c0_dev, ic0) || upload_owned(T0, &B.inst_c1_dev, ic1) ||
        upload_owned(T0, &B.ticket_dev, std::vector<int>(ninst, 0)) ||
        upload_owned(T0, &B.partial_dev, std::vector<double>(size_t(B.nchunks_all) * s, 0.0)))
      return 1;
  }
  GMG_CHECK(pack_off[ninst] < (1LL << 31), "batched hierarchy: more than 2^31 top-level rows");
  Level &T = mg->lev.back();
  GMG_CUDA(cudaMalloc(&B.conv_dev, ninst));
  T.own.push_back(B.conv_dev);
  GMG_CUDA(cudaMemset(B.conv_dev, 0, ninst));
  GMG_CUDA(cudaMallocHost(&B.conv_host, ninst));
  std::memset(B.conv_host, 0, ninst);
  GMG_CUDA(cudaMalloc(&B.norms_dev, sizeof(double) * ninst * GMG_MAX_S));
  T.own.push_back(B.norms_dev);
  GMG_CUDA(cudaMemset(B.norms_dev, 0, sizeof(double) * ninst * GMG_MAX_S));
  GMG_CUDA(cudaMallocHost(&B.norms_host, sizeof(double) * ninst * GMG_MAX_S));
  *out = mg.release();
  return 0;
}

int gmg_mg_num_instances(const gmg_mg *mg) { return mg ? mg->batch.ninst : 0; }

int gmg_mg_instance_info(const gmg_mg *mg, int k, int *top, int *n_top, long long *pack_offset) {
  if (!mg || k < 0 || k >= mg->batch.ninst) { set_error("gmg_mg_instance_info: bad instance %d", k); return 1; }
  if (top) *top = mg->batch.top[k];
  if (n_top) *n_top = mg->batch.nrows_top[k];
  if (pack_offset) *pack_offset = mg->batch.pack_off[k];
  return 0;
}

int gmg_mg_destroy(gmg_mg *mg) {
  delete mg;
  return 0;
}

int gmg_mg_set_stream(gmg_mg *mg, void *stream) {
  if (!mg) return 1;
  if (mg->own_stream && mg->stream) cudaStreamDestroy(mg->stream);
  mg->own_stream = false;
  mg->stream = (cudaStream_t)stream;
  return 0;
}

int gmg_mg_nlevels(const gmg_mg *mg) { return mg ? int(mg->lev.size()) : 0; }

int gmg_mg_level_size(const gmg_mg *mg, int level, int *n, int *s, long long *nnzb) {
  if (!mg || level < 0 || level >= (int)mg->lev.size()) { set_error("bad level"); return 1; }
  const Level &L = mg->lev[level];
  if (n) *n = L.n;
  if (s) *s = L.s;
  if (nnzb) *nnzb = L.nnzb;
  return 0;
}

int gmg_mg_get_order(const gmg_mg *mg, int level, int *perm) {
  if (!mg || level < 0 || level >= (int)mg->lev.size()) { set_error("bad level"); return 1; }
  std::copy(mg->lev[level].perm.begin(), mg->lev[level].perm.end(), perm);
  return 0;
}

int gmg_mg_get_matrix(const gmg_mg *mg, int level, int *rowptr, int *col, double *val) {
  if (!mg || level < 0 || level >= (int)mg->lev.size()) { set_error("bad level"); return 1; }
  const Level &L = mg->lev[level];
  if (rowptr) std::copy(L.h_rowptr.begin(), L.h_rowptr.end(), rowptr);
  if (col) std::copy(L.h_col.begin(), L.h_col.end(), col);
  if (val) std::copy(L.h_val.begin(), L.h_val.end(), val);
  return 0;
}

int gmg_mg_set_direct_host(gmg_mg *mg, int on) {
  if (!mg || (on != 0 && on != 1)) {
    set_error("gmg_mg_set_direct_host: bad arguments");
    return 1;
  }
  if (on) {
    int v = 0;
    GMG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, mg->device));
    GMG_CHECK(v, "gmg_mg_set_direct_host: the device does not read pageable host memory through the host page tables");
  }
  mg->direct_host = on != 0;
  return 0;
}

int gmg_mg_set_iface_sweep(gmg_mg *mg, int mode) {
  if (!mg || mode < 0 || mode > 2) {
    set_error("gmg_mg_set_iface_sweep: bad arguments");
    return 1;
  }
  mg->iface_sweep = mode;
  return 0;
}

int gmg_colour_graph(int n, const int *rowptr, const int *col, int *colour, int *ncolours) {
  if (n < 0 || (n > 0 && (!rowptr || !col || !colour)) || !ncolours) {
    set_error("gmg_colour_graph: bad arguments");
    return 1;
  }
  for (int i = 0; i < n; ++i)
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (col[k] < 0 || col[k] >= n) {
        set_error("gmg_colour_graph: row %d: column %d out of range", i, col[k]);
        return 1;
      }
  int nc = 0;
  const std::vector<int> c = colour_graph(n, sym_adjacency(n, rowptr, col), &nc);
  std::copy(c.begin(), c.end(), colour);
  *ncolours = nc;
  return 0;
}

int gmg_mg_domain_info(const gmg_mg *mg, int level, int *nsub, int *ninterior, int *ncolours) {
  if (!mg || level < 0 || level >= (int)mg->lev.size() || !nsub || !ninterior || !ncolours) {
    set_error("gmg_mg_domain_info: bad arguments");
    return 1;
  }
  const Level &L = mg->lev[level];
  *nsub = L.dom_nreg;
  *ninterior = L.dom_nint;
  *ncolours = L.dom_cptr.empty() ? 0 : int(L.dom_cptr.size()) - 1;
  return 0;
}

int gmg_mg_num_waves(const gmg_mg *mg, int level) {
  if (!mg || level < 0 || level >= (int)mg->lev.size()) return -1;
  return mg->lev[level].lower.nwave();
}

long long gmg_mg_device_bytes(const gmg_mg *mg) {
  if (!mg) return 0;
  long long b = 0;
  for (const auto &L : mg->lev) b += (long long)L.arena.size;
  for (auto &kv : mg->vecs)
    for (size_t l = 0; l < kv.second->lev.size(); ++l)
      b += (long long)mg->lev[l].n * mg->lev[l].s * (kv.second->prec == GMG_PREC_FP64 ? 8 : 4);
  return b;
}

long long gmg_mg_launch_count(const gmg_mg *mg, int reset) {
  if (!mg) return 0;
  long long c = mg->launches;
  if (reset) const_cast<gmg_mg *>(mg)->launches = 0;
  return c;
}

int gmg_mg_sync(gmg_mg *mg) {
  if (!mg) return 1;
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  GMG_CUDA(cudaGetLastError());
  // a one-launch interface ILU sweep whose completion wait ran out (its rows
  // became NaN): report it once and clear the flag
  for (size_t l = 0; l < mg->lev.size(); ++l) {
    const Level &L = mg->lev[l];
    if (!L.iface_err) continue;
    int e = 0;
    GMG_CUDA(cudaMemcpy(&e, L.iface_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
      GMG_CUDA(cudaMemset(L.iface_err, 0, sizeof(int)));
      set_error("level %zu: an interface ILU sweep gave up waiting for a neighbour row (results are NaN)", l);
      return 1;
    }
  }
  return 0;
}

}  // extern "C"
