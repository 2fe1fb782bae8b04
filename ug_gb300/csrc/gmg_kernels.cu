// CUDA kernels of the lmgc hot path for GB300 (sm_103a).
//
// Every kernel is a memory-bound sparse or vector pass; none of them maps to
// tensor cores.  Layout: block-CSR in processing order, 256-byte aligned
// arrays in one arena.  Rows are handled by groups of TPR consecutive threads
// (TPR = threads per row) so that a warp reads 32 consecutive (column,
// value) pairs -- coalesced -- and the TPR partial sums are combined with
// warp shuffles.  Block sizes S = 1, 2, 3 are compiled as templates so every
// block product is unrolled in registers.
//
// The arithmetic of each kernel follows the UG routine named in its comment;
// results agree with the reference to rounding (the summation order inside a
// row follows the shuffle tree instead of the MATRIX list).
#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <utility>

#include "gmg_internal.h"

namespace gmg {

namespace {

constexpr int BLK = 256;

// Programmatic dependent launch: every kernel is launched with programmatic
// stream serialisation, waits for its predecessor's memory before touching
// any data (griddepcontrol.wait) and immediately allows its successor to be
// launched (griddepcontrol.launch_dependents), so the successor's launch
// and scheduling overlap this kernel's tail.  Without the launch attribute
// both instructions are no-ops.
__device__ __forceinline__ void pdl_prologue() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

// Kernels whose matrix structure is constant for the hierarchy's lifetime
// load it BEFORE waiting for their predecessor (the loads overlap the
// predecessor's tail), then wait, then let their successor launch, so only
// the gathers of data the predecessor wrote remain on the dependent chain.
// The successor is launched only after this kernel's wait, so at most two
// kernels of the stream are ever resident at once.
__device__ __forceinline__ void pdl_wait_then_trigger() { pdl_prologue(); }

// entries of a row prefetched before the wait.  Only launches of at most
// PREFETCH_MAX_BLOCKS blocks use the prefetching variants (PN > 0): those
// are latency-bound, while on larger grids the extra registers cost more
// occupancy than the overlap gains, and the plain streaming loop (PN = 0) is
// faster.
template <int S>
struct PF {
  static constexpr int N = S == 1 ? 16 : (S == 2 ? 7 : 4);
};
constexpr long long PREFETCH_MAX_BLOCKS = 1100;  // ~280k rows (measured: the 65^3 level gains, 320k+ rows lose)

// PN < 0 selects the plain loop with evict-first loads of the matrix stream
// (ld.global.cs): used where a level's sliced-ELLPACK matrix is larger than
// most of L2, so that its single-use stream does not push out the gathered
// vector entries; smaller matrices keep the default policy, which lets them
// stay in L2 from one smoothing step to the next.
constexpr long long STREAM_MIN_BYTES = 96ll << 20;

// per-level variant choice: the autotuner's (Level::prefetch / Level::stream
// 0 or 1), else the thresholds above (-1)
inline bool use_prefetch(const Level &L, long long grid) {
  return L.prefetch < 0 ? grid <= PREFETCH_MAX_BLOCKS : L.prefetch != 0;
}
constexpr long long REFINE_STREAM_MIN_BYTES = 16ll << 20;
inline bool use_stream(const Level &L, long long bytes) { return L.stream < 0 ? bytes > STREAM_MIN_BYTES : L.stream != 0; }
template <bool ST, class T>
__device__ __forceinline__ T ld_mat(const T *p) {
  if constexpr (ST) return __ldcs(p);
  else return __ldg(p);
}

// a sliced-ELLPACK row i: entry k at e0 + 32 k, w entries (padding included);
// the first PF<S>::N (column, block) pairs are held in registers
template <class T, int S, int P_ = PF<S>::N>
struct SellRow {
  static constexpr int P = P_;
  int e0, w;
  int col[P > 0 ? P : 1];
  T val[P > 0 ? P : 1][S * S];
  __device__ __forceinline__ void load(int i, const int *__restrict__ sptr, const int *__restrict__ scol,
                                       const T *__restrict__ sval) {
    const int base = __ldg(sptr + (i >> 5));
    w = (__ldg(sptr + (i >> 5) + 1) - base) >> 5;
    e0 = base + (i & 31);
#pragma unroll
    for (int k = 0; k < P; ++k) {
      col[k] = 0;
      if (k < w) {
        const int e = e0 + 32 * k;
        col[k] = __ldg(scol + e);
#pragma unroll
        for (int q = 0; q < S * S; ++q) val[k][q] = __ldg(sval + (size_t)e * (S * S) + q);
      }
    }
  }
};

// entries kb..ke-1 of sliced-ELLPACK row i (e0 = entry kb, w = ke - kb); the
// first P held in registers.  Rows of a split level (Level::sell_split) store
// the diagonal, their sell_nl[i] strictly lower blocks, then the upper ones:
// part 0 = all off-diagonal entries, 1 = the lower ones, 2 = the upper ones
// and the padding.  Unsplit levels keep every off-diagonal entry in each part
// (the kernels test the column).
template <class T, int S, int P_>
struct SellPart {
  static constexpr int P = P_;
  int e0, w;
  int col[P > 0 ? P : 1];
  T val[P > 0 ? P : 1][S * S];
  // the w entries from entry e0_ on (their start already known)
  __device__ __forceinline__ void load_at(int e0_, int w_, const int *__restrict__ scol, const T *__restrict__ sval) {
    e0 = e0_;
    w = w_;
#pragma unroll
    for (int k = 0; k < P; ++k) {
      col[k] = 0;
      if (k < w) {
        const int e = e0 + 32 * k;
        col[k] = __ldg(scol + e);
#pragma unroll
        for (int q = 0; q < S * S; ++q) val[k][q] = __ldg(sval + (size_t)e * (S * S) + q);
      }
    }
  }
  __device__ __forceinline__ void load(int i, int part, const int *__restrict__ sptr, const uint8_t *__restrict__ nl,
                                       const int *__restrict__ scol, const T *__restrict__ sval) {
    const int base = __ldg(sptr + (i >> 5));
    const int wt = (__ldg(sptr + (i >> 5) + 1) - base) >> 5;
    int kb = 1, ke = wt;
    if (nl && part) {
      const int m = 1 + __ldg(nl + i);
      if (part == 1) ke = m;
      else kb = m;
    }
    w = ke - kb;
    e0 = base + (i & 31) + 32 * kb;
#pragma unroll
    for (int k = 0; k < P; ++k) {
      col[k] = 0;
      if (k < w) {
        const int e = e0 + 32 * k;
        col[k] = __ldg(scol + e);
#pragma unroll
        for (int q = 0; q < S * S; ++q) val[k][q] = __ldg(sval + (size_t)e * (S * S) + q);
      }
    }
  }
};

template <typename... KP, typename... A>
inline void pdl_launch(gmg_mg *mg, void (*kern)(KP...), dim3 grid, dim3 block, A &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = mg->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = mg->opts.disable_pdl ? 0 : 1;
  cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}
#define GMG_LAUNCH(K, G, B, ...) pdl_launch(mg, K, dim3(G), dim3(B), __VA_ARGS__)

// the same with dynamic shared memory (at most the default 48 KB)
template <typename... KP, typename... A>
inline void pdl_launch_smem(gmg_mg *mg, void (*kern)(KP...), dim3 grid, dim3 block, size_t smem, A &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = mg->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = mg->opts.disable_pdl ? 0 : 1;
  cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}

// the CSR entries k0 + lane + TPR q (q < Q) of one row held by one lane,
// prefetched before the wait
template <class T, int S, int Q>
struct CsrLane {
  int k1, col[Q > 0 ? Q : 1];
  T val[Q > 0 ? Q : 1][S * S];
  __device__ __forceinline__ void load(bool valid, int k0, int k1_, int lane, int tpr, const int *__restrict__ cols,
                                       const T *__restrict__ vals) {
    k1 = valid ? k1_ : 0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int k = k0 + lane + tpr * q;
      col[q] = 0;
      if (k < k1) {
        col[q] = __ldg(cols + k);
#pragma unroll
        for (int e = 0; e < S * S; ++e) val[q][e] = __ldg(vals + (size_t)k * (S * S) + e);
      }
    }
  }
};

template <class T>
struct Damp {
  T d[GMG_MAX_S];
};

template <class T>
Damp<T> make_damp(const double *damp, int s) {
  Damp<T> r;
  for (int i = 0; i < GMG_MAX_S; ++i) r.d[i] = T(damp ? damp[i < s ? i : 0] : 1.0);
  return r;
}

inline unsigned grid_for(long long threads) {
  long long g = (threads + BLK - 1) / BLK;
  return unsigned(g < 1 ? 1 : g);
}

template <int TPR, class T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
  for (int off = TPR / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// ------------------------------------------------------------ BLAS-1 kernels
template <class T>
__global__ void set_kernel(T *x, long long len, T a) {
  pdl_prologue();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    x[i] = a;
}
template <class T>
__global__ void copy_kernel(T *x, const T *__restrict__ y, long long len) {
  pdl_prologue();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    x[i] = y[i];
}
template <class T>
__global__ void add_kernel(T *x, const T *__restrict__ y, long long len) {
  pdl_prologue();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    x[i] += y[i];
}
template <class TD, class TS>
__global__ void convert_kernel(TD *x, const TS *__restrict__ y, long long len) {
  pdl_prologue();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    x[i] = TD(y[i]);
}
__global__ void refine_prepare_kernel(float *b32, float *c32, const double *__restrict__ b64, long long len) {
  pdl_prologue();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    b32[i] = float(b64[i]);
    c32[i] = 0.0f;
  }
}
template <class TS>
__global__ void add_mixed_kernel(double *x, const TS *__restrict__ y, long long len) {
  pdl_prologue();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    x[i] += double(y[i]);
}
// dscalx: x_i,r *= damp_r
template <class T, int S>
__global__ void scale_kernel(T *x, int n, Damp<T> dm) {
  pdl_prologue();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int r = 0; r < S; ++r) x[(size_t)i * S + r] *= dm.d[r];
}

// ------------------------------------------------------------ dmatmul_minus
// ugblas.cc:3997: x -= A y, row sums formed before the subtraction.
// ACC: additionally acc += y (the lmgc `dadd(c, t)` that follows every
// smoothing step and the coarse-grid correction, iter.cc:7811-7816, 7903).
template <class T, class TY, int S, int TPR, bool ACC, int Q>
__global__ void __launch_bounds__(BLK) spmv_minus_kernel(int n, const int *__restrict__ rowptr,
                                                         const int *__restrict__ col, const T *__restrict__ val,
                                                         const TY *__restrict__ y, T *__restrict__ x,
                                                         TY *__restrict__ acc) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = gt / TPR, lane = gt & (TPR - 1);
  const int k0 = row < n ? __ldg(rowptr + row) : 0, k1 = row < n ? __ldg(rowptr + row + 1) : 0;
  CsrLane<T, S, Q> E;
  E.load(row < n, k0, k1, lane, TPR, col, val);
  pdl_wait_then_trigger();
  T s[S];
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = T(0);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    if (k0 + lane + TPR * q < E.k1) {
      T yv[S];
#pragma unroll
      for (int c = 0; c < S; ++c) yv[c] = T(y[(size_t)E.col[q] * S + c]);
#pragma unroll
      for (int r = 0; r < S; ++r)
#pragma unroll
        for (int c = 0; c < S; ++c) s[r] = fma(E.val[q][r * S + c], yv[c], s[r]);
    }
  }
  for (int k = k0 + lane + TPR * Q; k < E.k1; k += TPR) {
    const int j = __ldg(col + k);
    const T *m = val + (size_t)k * (S * S);
    T yv[S];
#pragma unroll
    for (int c = 0; c < S; ++c) yv[c] = T(y[(size_t)j * S + c]);
#pragma unroll
    for (int r = 0; r < S; ++r)
#pragma unroll
      for (int c = 0; c < S; ++c) s[r] = fma(__ldg(m + r * S + c), yv[c], s[r]);
  }
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = group_sum<TPR>(s[r]);
  if (row < n && lane == 0) {
#pragma unroll
    for (int r = 0; r < S; ++r) {
      x[(size_t)row * S + r] -= s[r];
      if (ACC) acc[(size_t)row * S + r] += y[(size_t)row * S + r];
    }
  }
}

// Sliced-ELLPACK dmatmul_minus: one thread per row; entry k of the 32 rows
// of a slice are adjacent, so a warp loads 32 consecutive columns and values
// per step, all loads of a row are independent (no row-pointer chain, no
// shuffle reduction: one FMA per stored entry, which matters for FP64 on
// GB300).  Padding entries are zero blocks at the row itself.  (Loading a
// row's column indices in one predicated batch before the gathers measured
// slower on GB300 than this plain loop, which the compiler pipelines.)
template <class T, class TY, class TA, int S, bool ACC, int PN>
__global__ void __launch_bounds__(BLK) sell_spmv_kernel(int n, const int *__restrict__ sptr,
                                                        const int *__restrict__ scol, const T *__restrict__ sval,
                                                        const TY *__restrict__ y, T *__restrict__ x,
                                                        TA *__restrict__ acc) {
  constexpr int P0 = PN > 0 ? PN : 0;
  constexpr bool ST = PN < 0;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  SellRow<T, S, P0> R;
  R.load(i, sptr, scol, sval);
  pdl_wait_then_trigger();
  T s[S];
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = T(0);
#pragma unroll
  for (int k = 0; k < P0; ++k) {
    if (k < R.w) {
#pragma unroll
      for (int c = 0; c < S; ++c) {
        const T yv = T(y[(size_t)R.col[k] * S + c]);
#pragma unroll
        for (int r = 0; r < S; ++r) s[r] = fma(R.val[k][r * S + c], yv, s[r]);
      }
    }
  }
  int e = R.e0 + 32 * P0;
#pragma unroll 4
  for (int k = P0; k < R.w; ++k, e += 32) {
    const int j = ld_mat<ST>(scol + e);
    const T *m = sval + (size_t)e * (S * S);
#pragma unroll
    for (int c = 0; c < S; ++c) {
      const T yv = T(y[(size_t)j * S + c]);
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = fma(ld_mat<ST>(m + r * S + c), yv, s[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < S; ++r) {
    x[(size_t)i * S + r] -= s[r];
    if (ACC) acc[(size_t)i * S + r] += TA(y[(size_t)i * S + r]);
  }
}

// Sliced-ELLPACK l_lgs wave over the contiguous rows [r0, r1) of one colour:
// entries to rows j < i (earlier colours) are final, the diagonal (entry 0)
// and the padding (j == i) are skipped.
template <class T, int S, bool ALL_ACTIVE, int PN>
__global__ void __launch_bounds__(BLK) sell_gs_kernel(int r0, int r1, const int *__restrict__ sptr,
                                                      const uint8_t *__restrict__ nl, const int *__restrict__ scol,
                                                      const T *__restrict__ sval, const T *__restrict__ dinv,
                                                      const uint8_t *__restrict__ flags, const T *__restrict__ b,
                                                      T *__restrict__ t) {
  const int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1) return;
  const bool act = ALL_ACTIVE || (__ldg(flags + i) & F_ACTIVE);
  SellPart<T, S, PN> R;
  T D[S * S];
  if (act) {
    R.load(i, 1, sptr, nl, scol, sval);
#pragma unroll
    for (int q = 0; q < S * S; ++q) D[q] = __ldg(dinv + (size_t)i * S * S + q);
  }
  pdl_wait_then_trigger();
  if (!act) {
#pragma unroll
    for (int r = 0; r < S; ++r) t[(size_t)i * S + r] = T(0);
    return;
  }
  T s[S];
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = b[(size_t)i * S + r];
#pragma unroll
  for (int k = 0; k < PN; ++k) {
    if (k < R.w && R.col[k] < i) {
#pragma unroll
      for (int c = 0; c < S; ++c) {
        const T tv = t[(size_t)R.col[k] * S + c];
#pragma unroll
        for (int r = 0; r < S; ++r) s[r] = fma(-R.val[k][r * S + c], tv, s[r]);
      }
    }
  }
  int e = R.e0 + 32 * (PN > 0 ? PN : 0);
#pragma unroll 4
  for (int k = PN > 0 ? PN : 0; k < R.w; ++k, e += 32) {
    const int j = __ldg(scol + e);
    if (j >= i) continue;
    const T *m = sval + (size_t)e * (S * S);
#pragma unroll
    for (int c = 0; c < S; ++c) {
      const T tv = t[(size_t)j * S + c];
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = fma(-__ldg(m + r * S + c), tv, s[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < S; ++r) {
    T v = T(0);
#pragma unroll
    for (int c = 0; c < S; ++c) v = fma(D[r * S + c], s[c], v);
    t[(size_t)i * S + r] = v;
  }
}

// ------------------------------------------------------------ chained Gauss-Seidel steps
// nu multicolour Gauss-Seidel smoothing steps of lmgc (Step, dadd(c, t),
// b -= A t each) with the defect kept implicit between steps: after a step
// (D+L) t = b, so the new defect is b - A t = -U t.  Step 1 of a wave row i:
// t_i = D_i^{-1}(b_i - sum_{j<i} a_ij t_j); later steps: t_i = D_i^{-1}(
// -sum_{j != i} a_ij t_j), t updated in place (rows of earlier colours hold
// the new t, later colours still the previous one); each step adds t to c.
// After the last step sell_upper_defect_kernel writes b = -U t.  Exact in
// real arithmetic; rounding differs from the step-by-step form.  Only for
// all-ACTIVE levels, unit damping and colour-contiguous waves.
template <class T, int S, bool FIRST, int PN>
__global__ void __launch_bounds__(BLK) sell_gs_chain_kernel(int r0, int r1, const int *__restrict__ sptr,
                                                            const uint8_t *__restrict__ nl,
                                                            const int *__restrict__ scol, const T *__restrict__ sval,
                                                            const T *__restrict__ dinv, const T *__restrict__ b,
                                                            T *__restrict__ t, T *__restrict__ c) {
  const int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1) return;
  SellPart<T, S, PN> R;
  T D[S * S];
  R.load(i, FIRST ? 1 : 0, sptr, nl, scol, sval);
#pragma unroll
  for (int q = 0; q < S * S; ++q) D[q] = __ldg(dinv + (size_t)i * S * S + q);
  pdl_wait_then_trigger();
  T s[S];
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = FIRST ? b[(size_t)i * S + r] : T(0);
#pragma unroll
  for (int k = 0; k < PN; ++k) {
    if (k < R.w && (FIRST ? R.col[k] < i : R.col[k] != i)) {
#pragma unroll
      for (int cc = 0; cc < S; ++cc) {
        const T tv = t[(size_t)R.col[k] * S + cc];
#pragma unroll
        for (int r = 0; r < S; ++r) s[r] = fma(-R.val[k][r * S + cc], tv, s[r]);
      }
    }
  }
  int e = R.e0 + 32 * (PN > 0 ? PN : 0);
#pragma unroll 4
  for (int k = PN > 0 ? PN : 0; k < R.w; ++k, e += 32) {
    const int j = __ldg(scol + e);
    if (FIRST ? j >= i : j == i) continue;
    const T *m = sval + (size_t)e * (S * S);
#pragma unroll
    for (int cc = 0; cc < S; ++cc) {
      const T tv = t[(size_t)j * S + cc];
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = fma(-__ldg(m + r * S + cc), tv, s[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < S; ++r) {
    T v = T(0);
#pragma unroll
    for (int cc = 0; cc < S; ++cc) v = fma(D[r * S + cc], s[cc], v);
    t[(size_t)i * S + r] = v;
    c[(size_t)i * S + r] += v;
  }
}

// b = -U t: the defect after the last chained step (entries j > i)
template <class T, int S, int PN>
__global__ void __launch_bounds__(BLK) sell_upper_defect_kernel(int n, const int *__restrict__ sptr,
                                                                const uint8_t *__restrict__ nl,
                                                                const int *__restrict__ scol,
                                                                const T *__restrict__ sval, const T *__restrict__ t,
                                                                T *__restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  SellPart<T, S, PN> R;
  R.load(i, 2, sptr, nl, scol, sval);
  pdl_wait_then_trigger();
  T s[S];
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = T(0);
#pragma unroll
  for (int k = 0; k < PN; ++k) {
    if (k < R.w && R.col[k] > i) {
#pragma unroll
      for (int cc = 0; cc < S; ++cc) {
        const T tv = t[(size_t)R.col[k] * S + cc];
#pragma unroll
        for (int r = 0; r < S; ++r) s[r] = fma(-R.val[k][r * S + cc], tv, s[r]);
      }
    }
  }
  int e = R.e0 + 32 * (PN > 0 ? PN : 0);
#pragma unroll 4
  for (int k = PN > 0 ? PN : 0; k < R.w; ++k, e += 32) {
    const int j = __ldg(scol + e);
    if (j <= i) continue;
    const T *m = sval + (size_t)e * (S * S);
#pragma unroll
    for (int cc = 0; cc < S; ++cc) {
      const T tv = t[(size_t)j * S + cc];
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = fma(-__ldg(m + r * S + cc), tv, s[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < S; ++r) b[(size_t)i * S + r] = s[r];
}

// ------------------------------------------------------------ chained steps in one block
// The chained steps and the closing b = -U t of one small sliced-ELLPACK
// level (a few thousand rows) run by ONE thread block. Each colour wave of a
// level that small keeps a few warps busy, and as separate launches every
// wave pays a kernel handoff (~1.3 us) plus an L2 gather. Here the waves are
// separated by __syncthreads. t and c live in shared memory for the whole
// call. The matrix streams from L2 in its sliced-ELLPACK layout. Each
// thread's first row of the next wave (and, in the first step, its b) is
// loaded before the barrier, so the barrier hides those loads. Every row does
// the arithmetic of sell_gs_chain_kernel / sell_upper_defect_kernel in the
// same order, so the results are bit-identical to the per-wave launches.
template <class T, int S, int PN, int NT>
__global__ void __launch_bounds__(NT, 1) sell_gs_chain_cta_kernel(const __grid_constant__ CtaWaves W,
                                                                  const int *__restrict__ sptr,
                                                                  const uint8_t *__restrict__ nl,
                                                                  const int *__restrict__ scol,
                                                                  const T *__restrict__ sval,
                                                                  const T *__restrict__ dinv, T *__restrict__ b,
                                                                  T *__restrict__ t, T *__restrict__ c) {
  extern __shared__ __align__(16) unsigned char cta_smem[];
  T *ts = reinterpret_cast<T *>(cta_smem);  // t, n * S
  T *cs = ts + (size_t)W.n * S;             // c, n * S
  const int tid = threadIdx.x;
  SellPart<T, S, PN> R;
  T D[S * S], bi[S];
  // the static part of a row: its entries of step st and its inverse diagonal
  auto load_row = [&](int i, int st) {
    R.load(i, st == 0 ? 1 : 0, sptr, nl, scol, sval);
#pragma unroll
    for (int q = 0; q < S * S; ++q) D[q] = __ldg(dinv + (size_t)i * S * S + q);
  };
  auto load_b = [&](int i) {
#pragma unroll
    for (int r = 0; r < S; ++r) bi[r] = b[(size_t)i * S + r];
  };
  int first = W.ptr[0] + tid;
  if (first < W.ptr[1]) load_row(first, 0);
  pdl_wait_then_trigger();
  for (int k = tid; k < W.n * S; k += NT) cs[k] = c[k];
  if (first < W.ptr[1]) load_b(first);
  __syncthreads();
  for (int st = 0; st < W.steps; ++st) {
    for (int w = 0; w < W.nwave; ++w) {
      const int r0 = W.ptr[w], r1 = W.ptr[w + 1];
      for (int i = r0 + tid; i < r1; i += NT) {
        if (i != r0 + tid) {
          load_row(i, st);
          if (st == 0) load_b(i);
        }
        T s[S];
#pragma unroll
        for (int r = 0; r < S; ++r) s[r] = st == 0 ? bi[r] : T(0);
#pragma unroll
        for (int k = 0; k < PN; ++k) {
          if (k < R.w && (st == 0 ? R.col[k] < i : R.col[k] != i)) {
#pragma unroll
            for (int cc = 0; cc < S; ++cc) {
              const T tv = ts[(size_t)R.col[k] * S + cc];
#pragma unroll
              for (int r = 0; r < S; ++r) s[r] = fma(-R.val[k][r * S + cc], tv, s[r]);
            }
          }
        }
        int e = R.e0 + 32 * (PN > 0 ? PN : 0);
        for (int k = PN > 0 ? PN : 0; k < R.w; ++k, e += 32) {
          const int j = __ldg(scol + e);
          if (st == 0 ? j >= i : j == i) continue;
          const T *m = sval + (size_t)e * (S * S);
#pragma unroll
          for (int cc = 0; cc < S; ++cc) {
            const T tv = ts[(size_t)j * S + cc];
#pragma unroll
            for (int r = 0; r < S; ++r) s[r] = fma(-__ldg(m + r * S + cc), tv, s[r]);
          }
        }
#pragma unroll
        for (int r = 0; r < S; ++r) {
          T v = T(0);
#pragma unroll
          for (int cc = 0; cc < S; ++cc) v = fma(D[r * S + cc], s[cc], v);
          ts[(size_t)i * S + r] = v;
          cs[(size_t)i * S + r] += v;
        }
      }
      // this thread's first row of the next wave, before the barrier
      const int w2 = w + 1 < W.nwave ? w + 1 : 0, st2 = w + 1 < W.nwave ? st : st + 1;
      const int i2 = W.ptr[w2] + tid;
      if (st2 < W.steps && i2 < W.ptr[w2 + 1]) {
        load_row(i2, st2);
        if (st2 == 0) load_b(i2);
      }
      __syncthreads();
    }
  }
  // b = -U t (unless the caller never reads it), then t and c back to global memory
  for (int i = tid; W.want_b && i < W.n; i += NT) {
    R.load(i, 2, sptr, nl, scol, sval);
    T s[S];
#pragma unroll
    for (int r = 0; r < S; ++r) s[r] = T(0);
#pragma unroll
    for (int k = 0; k < PN; ++k) {
      if (k < R.w && R.col[k] > i) {
#pragma unroll
        for (int cc = 0; cc < S; ++cc) {
          const T tv = ts[(size_t)R.col[k] * S + cc];
#pragma unroll
          for (int r = 0; r < S; ++r) s[r] = fma(-R.val[k][r * S + cc], tv, s[r]);
        }
      }
    }
    int e = R.e0 + 32 * (PN > 0 ? PN : 0);
    for (int k = PN > 0 ? PN : 0; k < R.w; ++k, e += 32) {
      const int j = __ldg(scol + e);
      if (j <= i) continue;
      const T *m = sval + (size_t)e * (S * S);
#pragma unroll
      for (int cc = 0; cc < S; ++cc) {
        const T tv = ts[(size_t)j * S + cc];
#pragma unroll
        for (int r = 0; r < S; ++r) s[r] = fma(-__ldg(m + r * S + cc), tv, s[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < S; ++r) b[(size_t)i * S + r] = s[r];
  }
  for (int k = tid; k < W.n * S; k += NT) {
    t[k] = ts[k];
    c[k] = cs[k];
  }
}

// ------------------------------------------------------------ chained steps in one cluster
// The same chained steps spread over a thread-block cluster of cw blocks on
// cw SMs.  Each colour wave is cut into chunks of 32 rows (one sliced-ELLPACK
// slice) dealt to the blocks in turn; a block's rows of a wave are numbered
// L = 0..cnt-1 and row L is done by thread L mod NT, its c_i kept in the
// block's slot of the row.  Every block holds the whole of t in its shared
// memory: a new t_i is stored into every block's copy through distributed
// shared memory, and the waves are separated by cluster barriers (release
// on arrive, acquire on wait).  With RS the matrix entries of the block's
// rows and their inverse diagonals are staged in its shared memory once per
// call (before the launch wait), so the waves read no global memory; without
// it only each row's inverse diagonal, first entry and widths are staged, the
// entries stream from L2, and each thread fetches its next row before it
// sends its new values.  The arithmetic of every row is that of
// sell_gs_chain_kernel, in the same order, so the results are bit-identical
// to the per-wave launches.
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
// the shared::cluster address of shared::cta address `a` in block q
__device__ __forceinline__ uint32_t cluster_map(uint32_t a, unsigned q) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(q));
  return r;
}
__device__ __forceinline__ void st_cluster(uint32_t a, float v) {
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}
__device__ __forceinline__ void st_cluster(uint32_t a, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}
// rows of a wave of len rows that block `rank` of cw takes (chunks rank,
// rank + cw, ...; the last chunk of the wave may be partial)
__host__ __device__ inline int cluster_share(int len, int cw, int rank) {
  const int nch = (len + 31) / 32;
  if (rank >= nch) return 0;
  const int mine = (nch - 1 - rank) / cw + 1;
  const int last = rank + (mine - 1) * cw;
  return (mine - 1) * 32 + (last == nch - 1 ? len - last * 32 : 32);
}
// the wave row of the block's row L: its chunk L / 32 is chunk (L / 32) cw + rank
__device__ __forceinline__ int cluster_row(int r0, int L, unsigned cw, unsigned rank) {
  return r0 + ((L >> 5) * int(cw) + int(rank)) * 32 + (L & 31);
}

template <class T, int S, int PN, int NT, bool RS>
__global__ void __launch_bounds__(NT, 1) sell_gs_chain_cluster_kernel(const __grid_constant__ CtaWaves W,
                                                                      const int *__restrict__ sptr,
                                                                      const uint8_t *__restrict__ nl,
                                                                      const int *__restrict__ scol,
                                                                      const T *__restrict__ sval,
                                                                      const T *__restrict__ dinv, T *__restrict__ b,
                                                                      T *__restrict__ t, T *__restrict__ c) {
  // t (n S) | c slots (own S) | inverse diagonals (own S S) | RS: values
  // (wm own S S), columns (wm own) | widths (own: off-diagonal entries |
  // lower ones << 16) | streamed: first off-diagonal entry (own) | first
  // slot of each wave (nwave + 1).  Slot q's entry k sits at k own + q.
  extern __shared__ __align__(16) unsigned char cl_smem[];
  T *ts = reinterpret_cast<T *>(cl_smem);
  T *cs = ts + (size_t)W.n * S;
  T *md = cs + (size_t)W.own * S;
  T *mv = md + (size_t)W.own * S * S;
  int *mc = reinterpret_cast<int *>(mv + (RS ? (size_t)W.wm * W.own * S * S : 0));
  int *mw = mc + (RS ? (size_t)W.wm * W.own : 0);
  int *me = mw + W.own;
  int *wb = me + (RS ? 0 : W.own);
  const uint32_t ts_sa = uint32_t(__cvta_generic_to_shared(ts));
  const unsigned cw = cluster_size(), rank = cluster_rank();
  const int tid = threadIdx.x;
  if (tid == 0) {
    int q = 0;
    for (int w = 0; w < W.nwave; ++w) {
      wb[w] = q;
      q += cluster_share(W.ptr[w + 1] - W.ptr[w], int(cw), int(rank));
    }
    wb[W.nwave] = q;
  }
  __syncthreads();
  const int nown = wb[W.nwave];
  // slot q of the block: its wave and row
  auto slot_row = [&](int q) {
    int w = 0;
    while (wb[w + 1] <= q) ++w;
    return cluster_row(W.ptr[w], q - wb[w], cw, rank);
  };
  // the entries kb..ke-1 (of the off-diagonal ones) of a part of slot q's
  // row: 0 all, 1 the lower, 2 the upper ones and the padding
  auto part_range = [&](int q, int part, int &kb, int &ke) {
    const int meta = mw[q], wt1 = meta & 0xffff, nlw = meta >> 16;
    kb = 0;
    ke = wt1;
    if (nl && part == 1) ke = nlw;
    if (nl && part == 2) kb = nlw;
  };
  // the static part of every slot's row, before the launch wait (slot q by
  // thread q mod NT)
  for (int q = tid; q < nown; q += NT) {
    const int i = slot_row(q);
    const int base = __ldg(sptr + (i >> 5));
    const int wt1 = ((__ldg(sptr + (i >> 5) + 1) - base) >> 5) - 1;
    mw[q] = wt1 | (nl ? int(__ldg(nl + i)) << 16 : 0);
#pragma unroll
    for (int z = 0; z < S * S; ++z) md[(size_t)q * S * S + z] = __ldg(dinv + (size_t)i * S * S + z);
    if constexpr (RS) {
      for (int k = 0; k < wt1; ++k) {
        const int e = base + (i & 31) + 32 * (k + 1);
        mc[(size_t)k * W.own + q] = __ldg(scol + e);
#pragma unroll
        for (int z = 0; z < S * S; ++z) mv[((size_t)k * W.own + q) * S * S + z] = __ldg(sval + (size_t)e * S * S + z);
      }
    } else {
      me[q] = base + (i & 31) + 32;
    }
  }
  SellPart<T, S, RS ? 1 : PN> R;
  T bi[S];
  auto load_row = [&](int q, int part) {
    if constexpr (!RS) {
      int kb, ke;
      part_range(q, part, kb, ke);
      R.load_at(me[q] + 32 * kb, ke - kb, scol, sval);
    }
  };
  auto load_b = [&](int i) {
#pragma unroll
    for (int r = 0; r < S; ++r) bi[r] = b[(size_t)i * S + r];
  };
  const int first = wb[1] > tid ? cluster_row(W.ptr[0], tid, cw, rank) : -1;
  if (first >= 0) load_row(tid, 1);  // slot tid, staged by this thread
  pdl_wait_then_trigger();
  for (int q = tid; q < nown; q += NT) {
    const int i = slot_row(q);
#pragma unroll
    for (int r = 0; r < S; ++r) cs[(size_t)q * S + r] = c[(size_t)i * S + r];
  }
  if (first >= 0) load_b(first);
  // every block has started and staged its rows before any stores into it
  cluster_arrive();
  cluster_wait();
  // s -= (a part of slot q's row) t, the entries failing the column test left out
  auto row_dot = [&](T *s, int i, int q, int st, int part) {
    if constexpr (RS) {
      int kb, ke;
      part_range(q, part, kb, ke);
      for (int k = kb; k < ke; ++k) {
        const int j = mc[(size_t)k * W.own + q];
        if (part == 2 ? j <= i : st == 0 ? j >= i : j == i) continue;
        const T *m = mv + ((size_t)k * W.own + q) * S * S;
#pragma unroll
        for (int cc = 0; cc < S; ++cc) {
          const T tv = ts[(size_t)j * S + cc];
#pragma unroll
          for (int r = 0; r < S; ++r) s[r] = fma(-m[r * S + cc], tv, s[r]);
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < PN; ++k) {
        if (k < R.w && (part == 2 ? R.col[k] > i : st == 0 ? R.col[k] < i : R.col[k] != i)) {
#pragma unroll
          for (int cc = 0; cc < S; ++cc) {
            const T tv = ts[(size_t)R.col[k] * S + cc];
#pragma unroll
            for (int r = 0; r < S; ++r) s[r] = fma(-R.val[k][r * S + cc], tv, s[r]);
          }
        }
      }
      int e = R.e0 + 32 * (PN > 0 ? PN : 0);
      for (int k = PN > 0 ? PN : 0; k < R.w; ++k, e += 32) {
        const int j = __ldg(scol + e);
        if (part == 2 ? j <= i : st == 0 ? j >= i : j == i) continue;
        const T *m = sval + (size_t)e * (S * S);
#pragma unroll
        for (int cc = 0; cc < S; ++cc) {
          const T tv = ts[(size_t)j * S + cc];
#pragma unroll
          for (int r = 0; r < S; ++r) s[r] = fma(-__ldg(m + r * S + cc), tv, s[r]);
        }
      }
    }
  };
  for (int st = 0; st < W.steps; ++st) {
    for (int w = 0; w < W.nwave; ++w) {
      const int r0 = W.ptr[w], cnt = wb[w + 1] - wb[w];
      // this thread's first row of the next wave, fetched while the new
      // values travel and the cluster gathers
      const int w2 = w + 1 < W.nwave ? w + 1 : 0, st2 = w + 1 < W.nwave ? st : st + 1;
      bool fetched = false;
      auto fetch_next = [&]() {
        fetched = true;
        if (st2 < W.steps && tid < wb[w2 + 1] - wb[w2]) {
          load_row(wb[w2] + tid, st2 == 0 ? 1 : 0);
          if (st2 == 0) load_b(cluster_row(W.ptr[w2], tid, cw, rank));
        }
      };
      for (int L = tid; L < cnt; L += NT) {
        const int i = cluster_row(r0, L, cw, rank), q = wb[w] + L;
        if (L != tid) {
          load_row(q, st == 0 ? 1 : 0);
          if (st == 0) load_b(i);
        }
        T s[S], v[S];
#pragma unroll
        for (int r = 0; r < S; ++r) s[r] = st == 0 ? bi[r] : T(0);
        row_dot(s, i, q, st, st == 0 ? 1 : 0);
#pragma unroll
        for (int r = 0; r < S; ++r) {
          v[r] = T(0);
#pragma unroll
          for (int cc = 0; cc < S; ++cc) v[r] = fma(md[(size_t)q * S * S + r * S + cc], s[cc], v[r]);
        }
        if (L + NT >= cnt) fetch_next();
#pragma unroll
        for (int r = 0; r < S; ++r) {
          const uint32_t off = ts_sa + uint32_t(((size_t)i * S + r) * sizeof(T));
          for (unsigned p = 0; p < cw; ++p) st_cluster(cluster_map(off, p), v[r]);
          cs[(size_t)q * S + r] += v[r];
        }
      }
      if (!fetched) fetch_next();
      cluster_arrive();
      cluster_wait();
    }
  }
  // b = -U t on the block's rows (unless the caller never reads it); t and c
  // back to global memory
  for (int q = tid; W.want_b && q < nown; q += NT) {
    const int i = slot_row(q);
    load_row(q, 2);
    T s[S];
#pragma unroll
    for (int r = 0; r < S; ++r) s[r] = T(0);
    row_dot(s, i, q, 1, 2);
#pragma unroll
    for (int r = 0; r < S; ++r) b[(size_t)i * S + r] = s[r];
  }
  for (int k = int(rank) * NT + tid; k < W.n * S; k += int(cw) * NT) t[k] = ts[k];
  for (int q = tid; q < nown; q += NT) {
    const int i = slot_row(q);
#pragma unroll
    for (int r = 0; r < S; ++r) c[(size_t)i * S + r] = cs[(size_t)q * S + r];
  }
}

// ------------------------------------------------------------ l_jac
// ugiter.cc:271: t = D^{-1} b on ACTIVE rows (0 elsewhere), then the
// smoother's dscalx by damp (iter.cc:836).  D^{-1} is stored per row.
template <class T, int S, bool ALL_ACTIVE>
__global__ void jac_kernel(int n, const T *__restrict__ dinv, const uint8_t *__restrict__ flags,
                           const T *__restrict__ b, T *__restrict__ t, Damp<T> dm) {
  pdl_prologue();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!ALL_ACTIVE && !(flags[i] & F_ACTIVE)) {
#pragma unroll
    for (int r = 0; r < S; ++r) t[(size_t)i * S + r] = T(0);
    return;
  }
  T bv[S];
#pragma unroll
  for (int c = 0; c < S; ++c) bv[c] = b[(size_t)i * S + c];
  const T *D = dinv + (size_t)i * S * S;
#pragma unroll
  for (int r = 0; r < S; ++r) {
    T v = T(0);
#pragma unroll
    for (int c = 0; c < S; ++c) v = fma(D[r * S + c], bv[c], v);
    t[(size_t)i * S + r] = v * dm.d[r];
  }
}

// ------------------------------------------------------------ fused Jacobi step
// One damped Jacobi smoothing step of lmgc in one pass: l_jac with the
// smoother's dscalx (t = damp D^{-1} b, 0 on rows that are not ACTIVE),
// dmatmul_minus (b -= A t) and dadd (c += t).  Every t_j is recomputed where
// it is used, from b_j and row j's inverse diagonal block with jac_kernel's
// arithmetic, so the results are those of the two-pass step.  The new defect
// goes to bout, which must not alias bin (rows read their neighbours' bin
// while others write).
template <class T, int S, bool ALL_ACTIVE>
__device__ __forceinline__ void jac_value(const T *__restrict__ dinv, const uint8_t *__restrict__ flags,
                                          const T *__restrict__ b, int j, const Damp<T> &dm, T *t) {
  if (!ALL_ACTIVE && !(__ldg(flags + j) & F_ACTIVE)) {
#pragma unroll
    for (int r = 0; r < S; ++r) t[r] = T(0);
    return;
  }
  T bv[S];
#pragma unroll
  for (int c = 0; c < S; ++c) bv[c] = __ldg(b + (size_t)j * S + c);
  const T *D = dinv + (size_t)j * S * S;
#pragma unroll
  for (int r = 0; r < S; ++r) {
    T v = T(0);
#pragma unroll
    for (int c = 0; c < S; ++c) v = fma(__ldg(D + r * S + c), bv[c], v);
    t[r] = v * dm.d[r];
  }
}

template <class T, int S, bool ALL_ACTIVE, int PN>
__global__ void __launch_bounds__(BLK) sell_jac_step_kernel(int n, const int *__restrict__ sptr,
                                                            const int *__restrict__ scol, const T *__restrict__ sval,
                                                            const T *__restrict__ dinv,
                                                            const uint8_t *__restrict__ flags,
                                                            const T *__restrict__ bin, T *__restrict__ bout,
                                                            T *__restrict__ c, Damp<T> dm) {
  constexpr int P0 = PN > 0 ? PN : 0;
  constexpr bool ST = PN < 0;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  SellRow<T, S, P0> R;
  R.load(i, sptr, scol, sval);
  pdl_wait_then_trigger();
  T s[S];
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = T(0);
#pragma unroll
  for (int k = 0; k < P0; ++k) {
    if (k < R.w) {
      T tv[S];
      jac_value<T, S, ALL_ACTIVE>(dinv, flags, bin, R.col[k], dm, tv);
#pragma unroll
      for (int cc = 0; cc < S; ++cc)
#pragma unroll
        for (int r = 0; r < S; ++r) s[r] = fma(R.val[k][r * S + cc], tv[cc], s[r]);
    }
  }
  int e = R.e0 + 32 * P0;
#pragma unroll 4
  for (int k = P0; k < R.w; ++k, e += 32) {
    const int j = ld_mat<ST>(scol + e);
    const T *m = sval + (size_t)e * (S * S);
    T tv[S];
    jac_value<T, S, ALL_ACTIVE>(dinv, flags, bin, j, dm, tv);
#pragma unroll
    for (int cc = 0; cc < S; ++cc)
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = fma(ld_mat<ST>(m + r * S + cc), tv[cc], s[r]);
  }
  T ti[S];
  jac_value<T, S, ALL_ACTIVE>(dinv, flags, bin, i, dm, ti);
#pragma unroll
  for (int r = 0; r < S; ++r) {
    bout[(size_t)i * S + r] = bin[(size_t)i * S + r] - s[r];
    c[(size_t)i * S + r] += ti[r];
  }
}

template <class T, int S, int TPR, bool ALL_ACTIVE>
__global__ void __launch_bounds__(BLK) jac_step_kernel(int n, const int *__restrict__ rowptr,
                                                       const int *__restrict__ col, const T *__restrict__ val,
                                                       const T *__restrict__ dinv, const uint8_t *__restrict__ flags,
                                                       const T *__restrict__ bin, T *__restrict__ bout,
                                                       T *__restrict__ c, Damp<T> dm) {
  pdl_prologue();
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = gt / TPR, lane = gt & (TPR - 1);
  T s[S];
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = T(0);
  if (row < n) {
    const int k1 = __ldg(rowptr + row + 1);
    for (int k = __ldg(rowptr + row) + lane; k < k1; k += TPR) {
      const int j = __ldg(col + k);
      const T *m = val + (size_t)k * (S * S);
      T tv[S];
      jac_value<T, S, ALL_ACTIVE>(dinv, flags, bin, j, dm, tv);
#pragma unroll
      for (int r = 0; r < S; ++r)
#pragma unroll
        for (int cc = 0; cc < S; ++cc) s[r] = fma(__ldg(m + r * S + cc), tv[cc], s[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = group_sum<TPR>(s[r]);
  if (row < n && lane == 0) {
    T ti[S];
    jac_value<T, S, ALL_ACTIVE>(dinv, flags, bin, row, dm, ti);
#pragma unroll
    for (int r = 0; r < S; ++r) {
      bout[(size_t)row * S + r] = bin[(size_t)row * S + r] - s[r];
      c[(size_t)row * S + r] += ti[r];
    }
  }
}

// ------------------------------------------------------------ l_lgs
// ugiter.cc:412: forward solve (D+L) t = b in processing order: row i uses
// the entries to rows j < i (VINDEX(w) < VINDEX(v)), all of which belong to
// earlier wavefronts and are final.  Inactive rows get 0.
template <class T, int S, int TPR, bool ALL_ACTIVE, int Q>
__global__ void __launch_bounds__(BLK) gs_wave_kernel(const int *__restrict__ rows, int nrows,
                                                      const int *__restrict__ rowptr, const int *__restrict__ col,
                                                      const T *__restrict__ val, const T *__restrict__ dinv,
                                                      const uint8_t *__restrict__ flags, const T *__restrict__ b,
                                                      T *__restrict__ t) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int idx = gt / TPR, lane = gt & (TPR - 1);
  const bool valid = idx < nrows;
  const int row = valid ? __ldg(rows + idx) : 0;
  const bool active = ALL_ACTIVE || (valid && (__ldg(flags + row) & F_ACTIVE));
  const bool work = valid && active;
  const int k0 = work ? __ldg(rowptr + row) + 1 : 0, k1 = work ? __ldg(rowptr + row + 1) : 0;
  CsrLane<T, S, Q> E;
  E.load(work, k0, k1, lane, TPR, col, val);
  pdl_wait_then_trigger();
  T s[S];
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = T(0);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    if (k0 + lane + TPR * q < E.k1 && E.col[q] < row) {
      T yv[S];
#pragma unroll
      for (int c = 0; c < S; ++c) yv[c] = t[(size_t)E.col[q] * S + c];
#pragma unroll
      for (int r = 0; r < S; ++r)
#pragma unroll
        for (int c = 0; c < S; ++c) s[r] = fma(E.val[q][r * S + c], yv[c], s[r]);
    }
  }
  for (int k = k0 + lane + TPR * Q; k < E.k1; k += TPR) {
    const int j = __ldg(col + k);
    if (j >= row) continue;
    const T *m = val + (size_t)k * (S * S);
    T yv[S];
#pragma unroll
    for (int c = 0; c < S; ++c) yv[c] = t[(size_t)j * S + c];
#pragma unroll
    for (int r = 0; r < S; ++r)
#pragma unroll
      for (int c = 0; c < S; ++c) s[r] = fma(__ldg(m + r * S + c), yv[c], s[r]);
  }
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = group_sum<TPR>(s[r]);
  if (valid && !active && lane == 0) {
#pragma unroll
    for (int r = 0; r < S; ++r) t[(size_t)row * S + r] = T(0);
  }
  if (work && lane == 0) {
    T rhs[S];
#pragma unroll
    for (int r = 0; r < S; ++r) rhs[r] = b[(size_t)row * S + r] - s[r];
    const T *D = dinv + (size_t)row * S * S;
#pragma unroll
    for (int r = 0; r < S; ++r) {
      T v = T(0);
#pragma unroll
      for (int c = 0; c < S; ++c) v = fma(D[r * S + c], rhs[c], v);
      t[(size_t)row * S + r] = v;
    }
  }
}

// ------------------------------------------------------------ l_luiter
// ugiter.cc:4444: forward with the unit lower factor, then backward with the
// strict upper factor and the stored inverse diagonal (StoreInverse).
// One wavefront of the ILU solve, TPR threads per row.  Each lane's first
// entry (column, factor block) and, backward, the inverse diagonal block are
// loaded before the launch wait (constant structure), so only the gathers of
// t written by the previous wavefront remain after it.
// DIAG: the rows have no upper-factor entries (the last colour of the
// subdomain order), so their backward step t = D^{-1} t follows at once
template <class T, int S, int TPR, bool ALL_ACTIVE, bool DIAG = false>
__global__ void __launch_bounds__(BLK) ilu_fwd_kernel(const int *__restrict__ rows, int nrows,
                                                      const int *__restrict__ rowptr, const int *__restrict__ col,
                                                      const T *__restrict__ val, const uint8_t *__restrict__ flags,
                                                      const T *__restrict__ b, T *__restrict__ t,
                                                      const T *__restrict__ dinv) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int idx = gt / TPR, lane = gt & (TPR - 1);
  const bool valid = idx < nrows;
  const int row = valid ? __ldg(rows + idx) : 0;
  const bool active = ALL_ACTIVE || (valid && (flags[row] & F_ACTIVE));
  int k = 0, k1 = 0, j0 = 0;
  T m0[S * S];
  if (valid && active) {
    k = __ldg(rowptr + row) + lane;
    k1 = __ldg(rowptr + row + 1);
    if (k < k1) {
      j0 = __ldg(col + k);
#pragma unroll
      for (int e = 0; e < S * S; ++e) m0[e] = __ldg(val + (size_t)k * (S * S) + e);
    }
  }
  pdl_prologue();
  T s[S];
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = T(0);
  if (k < k1) {
    T yv[S];
#pragma unroll
    for (int c = 0; c < S; ++c) yv[c] = t[(size_t)j0 * S + c];
#pragma unroll
    for (int r = 0; r < S; ++r)
#pragma unroll
      for (int c = 0; c < S; ++c) s[r] = fma(m0[r * S + c], yv[c], s[r]);
    for (k += TPR; k < k1; k += TPR) {
      const int j = __ldg(col + k);
      const T *m = val + (size_t)k * (S * S);
#pragma unroll
      for (int c = 0; c < S; ++c) yv[c] = t[(size_t)j * S + c];
#pragma unroll
      for (int r = 0; r < S; ++r)
#pragma unroll
        for (int c = 0; c < S; ++c) s[r] = fma(__ldg(m + r * S + c), yv[c], s[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = group_sum<TPR>(s[r]);
  if (valid && lane == 0) {
    if (DIAG && active) {
      T rhs[S];
#pragma unroll
      for (int r = 0; r < S; ++r) rhs[r] = b[(size_t)row * S + r] - s[r];
#pragma unroll
      for (int r = 0; r < S; ++r) {
        T v = T(0);
#pragma unroll
        for (int c = 0; c < S; ++c) v = fma(__ldg(dinv + (size_t)row * S * S + r * S + c), rhs[c], v);
        t[(size_t)row * S + r] = v;
      }
    } else {
#pragma unroll
      for (int r = 0; r < S; ++r) t[(size_t)row * S + r] = active ? b[(size_t)row * S + r] - s[r] : T(0);
    }
  }
}

// The interface part of the ILU solve in subdomain order, all colours of one
// direction in ONE cooperative launch.  Items are the interface rows colour
// after colour (forward 0..nc-1, backward nc-2..0), each colour padded to
// whole warps, TPR threads per row, grid-stride; a thread's rows never go
// back in colour, and no warp holds two colours.  A row whose factor entry
// points at an interface row solved in this launch waits for that row's
// completion flag (acquire; the writer stores t, then the flag with release
// semantics), reading t through L2.  Flags hold the launch's epoch + 1: the
// last block to finish advances the epoch, so flags are never reset.  Every
// row does ilu_fwd_kernel's / ilu_bwd_kernel's arithmetic in the same order
// (bit-identical).  A wait gives up after a bounded number of polls: the
// row's result becomes NaN (the ls loop's non-finite test then fails the
// solve) and *err is set.
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
constexpr int IFACE_MAX_POLLS = 1 << 16;

template <class T, int S, int TPR, bool ALL_ACTIVE, bool FWD>
__global__ void __launch_bounds__(BLK) ilu_iface_kernel(const int *__restrict__ items, int nitems, int nint,
                                                        int last_lo, const int *__restrict__ rowptr,
                                                        const int *__restrict__ col, const T *__restrict__ val,
                                                        const T *__restrict__ dinv, const uint8_t *__restrict__ flags,
                                                        const T *__restrict__ b, T *__restrict__ t,
                                                        unsigned *__restrict__ done, unsigned *__restrict__ ctr,
                                                        int *__restrict__ err) {
  const unsigned target = *(volatile unsigned *)ctr + 1u;
  const long long total = (long long)nitems * TPR, stride = (long long)gridDim.x * blockDim.x;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += stride) {
    const int q = int(g / TPR), lane = int(g & (TPR - 1));
    const int row = __ldg(items + q);
    const bool valid = row >= 0;
    const bool active = valid && (ALL_ACTIVE || (flags[row] & F_ACTIVE));
    bool ok = true;
    T s[S];
#pragma unroll
    for (int r = 0; r < S; ++r) s[r] = T(0);
    if (active) {
      const int k1 = __ldg(rowptr + row + 1);
      for (int k = __ldg(rowptr + row) + lane; k < k1; k += TPR) {
        const int j = __ldg(col + k);
        if (FWD ? j >= nint : j < last_lo) {  // solved in this launch
          int it = 0;
          while (ld_acquire_u32(done + (j - nint)) != target && ++it < IFACE_MAX_POLLS) __nanosleep(32);
          if (it >= IFACE_MAX_POLLS) ok = false;
        }
        const T *m = val + (size_t)k * (S * S);
        T yv[S];
#pragma unroll
        for (int c = 0; c < S; ++c) yv[c] = __ldcg(t + (size_t)j * S + c);
#pragma unroll
        for (int r = 0; r < S; ++r)
#pragma unroll
          for (int c = 0; c < S; ++c) s[r] = fma(__ldg(m + r * S + c), yv[c], s[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < S; ++r) s[r] = group_sum<TPR>(s[r]);
    ok = __all_sync(0xffffffffu, ok) != 0;  // the row group's lanes (whole warp: one colour)
    if (valid && lane == 0) {
      if (!ok) {
        atomicExch(err, 1);
#pragma unroll
        for (int r = 0; r < S; ++r) s[r] = T(NAN);
      }
      if (FWD) {
        if (row >= last_lo && active) {  // the last colour: no upper entries, backward step at once
          T rhs[S];
#pragma unroll
          for (int r = 0; r < S; ++r) rhs[r] = b[(size_t)row * S + r] - s[r];
#pragma unroll
          for (int r = 0; r < S; ++r) {
            T v = T(0);
#pragma unroll
            for (int c = 0; c < S; ++c) v = fma(__ldg(dinv + (size_t)row * S * S + r * S + c), rhs[c], v);
            t[(size_t)row * S + r] = v;
          }
        } else {
#pragma unroll
          for (int r = 0; r < S; ++r) t[(size_t)row * S + r] = active ? b[(size_t)row * S + r] - s[r] : T(0);
        }
      } else if (active) {
        T rhs[S];
#pragma unroll
        for (int r = 0; r < S; ++r) rhs[r] = __ldcg(t + (size_t)row * S + r) - s[r];
#pragma unroll
        for (int r = 0; r < S; ++r) {
          T v = T(0);
#pragma unroll
          for (int c = 0; c < S; ++c) v = fma(__ldg(dinv + (size_t)row * S * S + r * S + c), rhs[c], v);
          t[(size_t)row * S + r] = v;
        }
      }
      st_release_u32(done + (row - nint), target);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(ctr + 1, 1u) == gridDim.x - 1) {
      ctr[1] = 0;
      __threadfence();
      atomicAdd(ctr, 1u);
    }
  }
}

template <class T, int S, int TPR, bool ALL_ACTIVE>
__global__ void __launch_bounds__(BLK) ilu_bwd_kernel(const int *__restrict__ rows, int nrows,
                                                      const int *__restrict__ rowptr, const int *__restrict__ col,
                                                      const T *__restrict__ val, const T *__restrict__ dinv,
                                                      const uint8_t *__restrict__ flags, T *__restrict__ t) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int idx = gt / TPR, lane = gt & (TPR - 1);
  const bool valid = idx < nrows;
  const int row = valid ? __ldg(rows + idx) : 0;
  const bool work = valid && (ALL_ACTIVE || (flags[row] & F_ACTIVE));
  int k = 0, k1 = 0, j0 = 0;
  T m0[S * S], D[S * S];
  if (work) {
    k = __ldg(rowptr + row) + lane;
    k1 = __ldg(rowptr + row + 1);
    if (k < k1) {
      j0 = __ldg(col + k);
#pragma unroll
      for (int e = 0; e < S * S; ++e) m0[e] = __ldg(val + (size_t)k * (S * S) + e);
    }
    if (lane == 0)
#pragma unroll
      for (int e = 0; e < S * S; ++e) D[e] = __ldg(dinv + (size_t)row * S * S + e);
  }
  pdl_prologue();
  T s[S];
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = T(0);
  if (k < k1) {
    T yv[S];
#pragma unroll
    for (int c = 0; c < S; ++c) yv[c] = t[(size_t)j0 * S + c];
#pragma unroll
    for (int r = 0; r < S; ++r)
#pragma unroll
      for (int c = 0; c < S; ++c) s[r] = fma(m0[r * S + c], yv[c], s[r]);
    for (k += TPR; k < k1; k += TPR) {
      const int j = __ldg(col + k);
      const T *m = val + (size_t)k * (S * S);
#pragma unroll
      for (int c = 0; c < S; ++c) yv[c] = t[(size_t)j * S + c];
#pragma unroll
      for (int r = 0; r < S; ++r)
#pragma unroll
        for (int c = 0; c < S; ++c) s[r] = fma(__ldg(m + r * S + c), yv[c], s[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = group_sum<TPR>(s[r]);
  if (work && lane == 0) {
    T rhs[S];
#pragma unroll
    for (int r = 0; r < S; ++r) rhs[r] = t[(size_t)row * S + r] - s[r];
#pragma unroll
    for (int r = 0; r < S; ++r) {
      T v = T(0);
#pragma unroll
      for (int c = 0; c < S; ++c) v = fma(D[r * S + c], rhs[c], v);
      t[(size_t)row * S + r] = v;
    }
  }
}

// ILU sweep over the subdomain interiors of GMG_ORDER_DOMAIN: one block per
// subdomain walks its own wavefronts, separated by __syncthreads (an interior
// row has no neighbour outside its subdomain, so no other block's rows are
// involved; the interface rows run before (backward) or after (forward) as
// ordinary colour launches).  FWD: t = b - L t (unit lower factor), 0 off
// ACTIVE rows; backward: t = D^{-1} (t - U t) on ACTIVE rows.
constexpr int REGION_BLK = 128;
template <class T, int S, int TPR, bool ALL_ACTIVE, bool FWD>
__global__ void __launch_bounds__(REGION_BLK) ilu_region_kernel(
    const int *__restrict__ wbeg, const int *__restrict__ wptr, const int *__restrict__ rows,
    const int *__restrict__ rowptr, const int *__restrict__ col, const T *__restrict__ val, const T *__restrict__ dinv,
    const uint8_t *__restrict__ flags, const T *__restrict__ b, T *t) {
  pdl_prologue();
  const int w0 = __ldg(wbeg + blockIdx.x), w1 = __ldg(wbeg + blockIdx.x + 1);
  const int sub = threadIdx.x / TPR, lane = threadIdx.x & (TPR - 1);
  for (int w = w0; w < w1; ++w) {
    const int a = __ldg(wptr + w), e = __ldg(wptr + w + 1);
    for (int base = a; base < e; base += REGION_BLK / TPR) {
      const int idx = base + sub;
      const bool valid = idx < e;
      const int row = valid ? __ldg(rows + idx) : 0;
      const bool act = valid && (ALL_ACTIVE || (flags[row] & F_ACTIVE));
      T sm[S];
#pragma unroll
      for (int r = 0; r < S; ++r) sm[r] = T(0);
      if (act) {
        const int k1 = __ldg(rowptr + row + 1);
        for (int k = __ldg(rowptr + row) + lane; k < k1; k += TPR) {
          const int j = __ldg(col + k);
          const T *m = val + (size_t)k * (S * S);
          T yv[S];
#pragma unroll
          for (int c = 0; c < S; ++c) yv[c] = t[(size_t)j * S + c];
#pragma unroll
          for (int r = 0; r < S; ++r)
#pragma unroll
            for (int c = 0; c < S; ++c) sm[r] = fma(__ldg(m + r * S + c), yv[c], sm[r]);
        }
      }
#pragma unroll
      for (int r = 0; r < S; ++r) sm[r] = group_sum<TPR>(sm[r]);
      if (valid && lane == 0) {
        if (FWD) {
#pragma unroll
          for (int r = 0; r < S; ++r) t[(size_t)row * S + r] = act ? b[(size_t)row * S + r] - sm[r] : T(0);
        } else if (act) {
          T rhs[S];
#pragma unroll
          for (int r = 0; r < S; ++r) rhs[r] = t[(size_t)row * S + r] - sm[r];
          const T *D = dinv + (size_t)row * S * S;
#pragma unroll
          for (int r = 0; r < S; ++r) {
            T v = T(0);
#pragma unroll
            for (int c = 0; c < S; ++c) v = fma(D[r * S + c], rhs[c], v);
            t[(size_t)row * S + r] = v;
          }
        }
      }
    }
    __syncthreads();
  }
}

// The same sweep with the subdomain in shared memory: the block first copies
// its interior rows' right-hand side (forward) or current values (backward),
// the rows outside the interior it reads, its factor entries (local columns,
// values), the interior rows' entry ranges, ACTIVE flags and (backward)
// inverse diagonal blocks, and its wavefront bounds; the wavefronts then
// touch shared memory only, and the results are written back at the end.
// Dynamic shared memory, region_smem_bytes(): values (max_ent * S*S), inverse
// diagonals (max_rows * S*S, backward), vector entries (max_rows * S), then
// columns (max_ent), entry offsets (max_rows + 1), wave bounds
// (max_waves + 1) and flags (max_rows).
constexpr int REGION_TPR = 4;
template <class T, int S, bool ALL_ACTIVE, bool FWD>
__global__ void __launch_bounds__(REGION_BLK) ilu_region_smem_kernel(
    const int *__restrict__ wbeg, const int *__restrict__ wptr, const int *__restrict__ rows,
    const int *__restrict__ ent0, const int *__restrict__ lcol, const int *__restrict__ kidx,
    const int *__restrict__ ext0, const int *__restrict__ ext, const T *__restrict__ val, const T *__restrict__ dinv,
    const uint8_t *__restrict__ flags, const T *__restrict__ b, T *t, int max_ent, int max_rows) {
  constexpr int SS = S * S, TPR = REGION_TPR;
  extern __shared__ __align__(16) unsigned char region_smem[];
  T *v_s = reinterpret_cast<T *>(region_smem);
  T *d_s = v_s + (size_t)max_ent * SS;
  T *t_s = d_s + (FWD ? 0 : (size_t)max_rows * SS);
  int *c_s = reinterpret_cast<int *>(t_s + (size_t)max_rows * S);
  int *eo_s = c_s + max_ent;
  int *w_s = eo_s + max_rows + 1;
  const int r = blockIdx.x;
  const int wb = __ldg(wbeg + r), we = __ldg(wbeg + r + 1);
  uint8_t *a_s = reinterpret_cast<uint8_t *>(w_s + (we - wb) + 1);
  // structure first (constant for the hierarchy's lifetime), then the wait
  const int i0 = __ldg(wptr + wb), i1 = __ldg(wptr + we), nloc = i1 - i0;
  const int x0 = __ldg(ext0 + r), x1 = __ldg(ext0 + r + 1);
  const int e0 = __ldg(ent0 + i0), e1 = __ldg(ent0 + i1);
  for (int e = threadIdx.x; e < e1 - e0; e += blockDim.x) {
    c_s[e] = __ldg(lcol + e0 + e);
    const T *m = val + (size_t)__ldg(kidx + e0 + e) * SS;
#pragma unroll
    for (int q = 0; q < SS; ++q) v_s[e * SS + q] = __ldg(m + q);
  }
  for (int q = threadIdx.x; q <= nloc; q += blockDim.x) eo_s[q] = __ldg(ent0 + i0 + q) - e0;
  for (int w = threadIdx.x; w <= we - wb; w += blockDim.x) w_s[w] = __ldg(wptr + wb + w) - i0;
  for (int q = threadIdx.x; q < nloc; q += blockDim.x) {
    const int row = __ldg(rows + i0 + q);
    a_s[q] = ALL_ACTIVE || (flags[row] & F_ACTIVE);
    if (!FWD)
#pragma unroll
      for (int k = 0; k < SS; ++k) d_s[q * SS + k] = __ldg(dinv + (size_t)row * SS + k);
  }
  pdl_prologue();
  for (int q = threadIdx.x; q < nloc; q += blockDim.x) {
    const int row = __ldg(rows + i0 + q);
#pragma unroll
    for (int c = 0; c < S; ++c) t_s[q * S + c] = FWD ? b[(size_t)row * S + c] : t[(size_t)row * S + c];
  }
  for (int q = threadIdx.x; q < x1 - x0; q += blockDim.x) {
    const int row = __ldg(ext + x0 + q);
#pragma unroll
    for (int c = 0; c < S; ++c) t_s[(nloc + q) * S + c] = t[(size_t)row * S + c];
  }
  __syncthreads();
  const int sub = threadIdx.x / TPR, lane = threadIdx.x & (TPR - 1);
  for (int w = 0; w < we - wb; ++w) {
    const int a = w_s[w], e = w_s[w + 1];
    for (int base = a; base < e; base += REGION_BLK / TPR) {
      const int q = base + sub;
      const bool valid = q < e;
      const bool act = valid && a_s[q];
      T sm[S];
#pragma unroll
      for (int rr = 0; rr < S; ++rr) sm[rr] = T(0);
      if (act) {
        const int k1 = eo_s[q + 1];
        for (int k = eo_s[q] + lane; k < k1; k += TPR) {
          const int j = c_s[k];
          const T *m = v_s + k * SS;
#pragma unroll
          for (int rr = 0; rr < S; ++rr)
#pragma unroll
            for (int c = 0; c < S; ++c) sm[rr] = fma(m[rr * S + c], t_s[j * S + c], sm[rr]);
        }
      }
#pragma unroll
      for (int rr = 0; rr < S; ++rr) sm[rr] = group_sum<TPR>(sm[rr]);
      if (valid && lane == 0) {
        if (FWD) {
#pragma unroll
          for (int rr = 0; rr < S; ++rr) t_s[q * S + rr] = act ? t_s[q * S + rr] - sm[rr] : T(0);
        } else if (act) {
          T rhs[S];
#pragma unroll
          for (int rr = 0; rr < S; ++rr) rhs[rr] = t_s[q * S + rr] - sm[rr];
          const T *D = d_s + q * SS;
#pragma unroll
          for (int rr = 0; rr < S; ++rr) {
            T v = T(0);
#pragma unroll
            for (int c = 0; c < S; ++c) v = fma(D[rr * S + c], rhs[c], v);
            t_s[q * S + rr] = v;
          }
        }
      }
    }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < nloc; q += blockDim.x) {
    const int row = __ldg(rows + i0 + q);
#pragma unroll
    for (int c = 0; c < S; ++c) t[(size_t)row * S + c] = t_s[q * S + c];
  }
}

template <class T, int S>
size_t region_smem_bytes(const Level::RegionTab &R, bool fwd) {
  return (size_t(R.max_ent) * S * S + (fwd ? 0 : size_t(R.max_rows) * S * S) + size_t(R.max_rows) * S) * sizeof(T) +
         (size_t(R.max_ent) + R.max_rows + 1 + R.max_waves + 1) * sizeof(int) + size_t(R.max_rows);
}

// ------------------------------------------------------------ StandardRestrict
// transgrid.cc:117-232 as a gather over R = P^T: coarse rows with VNCLASS >= 2
// start from 0, the others keep their value; each contribution is
// weight * (damp * fine defect); components set in the coarse VECSKIP get none.
template <class T, int S, int PN>
__global__ void restrict_kernel(int nc, const int *__restrict__ rrow, const int *__restrict__ rcol,
                                const T *__restrict__ rw, const uint8_t *__restrict__ cflags,
                                const uint8_t *__restrict__ cskip, const T *__restrict__ from, T *__restrict__ to,
                                Damp<T> dm, T *__restrict__ zero) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  // the row of R (constant) before the wait
  constexpr int P = PN > 0 ? PN : 1;
  const int k0 = __ldg(rrow + c), k1 = __ldg(rrow + c + 1);
  int fc[P];
  T fw[P];
#pragma unroll
  for (int q = 0; q < PN; ++q) {
    fc[q] = 0;
    fw[q] = T(0);
    if (k0 + q < k1) {
      fc[q] = __ldg(rcol + k0 + q);
      fw[q] = __ldg(rw + k0 + q);
    }
  }
  const bool reset = __ldg(cflags + c) & F_RESET;
  const int sk = __ldg(cskip + c);
  pdl_wait_then_trigger();
  if (zero)  // lmgc's dset(c_{l-1}, 0), iter.cc:7873, in the same pass
#pragma unroll
    for (int r = 0; r < S; ++r) zero[(size_t)c * S + r] = T(0);
  T acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = reset ? T(0) : to[(size_t)c * S + r];
#pragma unroll
  for (int q = 0; q < PN; ++q)
    if (k0 + q < k1)
#pragma unroll
      for (int r = 0; r < S; ++r) acc[r] = fma(fw[q], dm.d[r] * from[(size_t)fc[q] * S + r], acc[r]);
  for (int k = k0 + PN; k < k1; ++k) {
    const int f = __ldg(rcol + k);
    const T w = __ldg(rw + k);
#pragma unroll
    for (int r = 0; r < S; ++r) acc[r] = fma(w, dm.d[r] * from[(size_t)f * S + r], acc[r]);
  }
#pragma unroll
  for (int r = 0; r < S; ++r)
    to[(size_t)c * S + r] = (sk & (1 << r)) ? (reset ? T(0) : to[(size_t)c * S + r]) : acc[r];
}

// ------------------------------------------------------------ StandardInterpolateCorrection
// transgrid.cc:235-347: t_f = sum_i (weight_i * damp) * c_i in every component
// the fine VECSKIP leaves free; rows skipped in all components stay 0.
template <class T, int S, bool ACC, int PN>
__global__ void interp_kernel(int nf, const int *__restrict__ prow, const int *__restrict__ pcol,
                              const T *__restrict__ pw, const uint8_t *__restrict__ fskip,
                              const T *__restrict__ from, T *__restrict__ to, Damp<T> dm, T *__restrict__ acc) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  // the row of P (constant) before the wait
  constexpr int P = PN > 0 ? PN : 1;
  const int sk = __ldg(fskip + f);
  const int k0 = __ldg(prow + f), k1 = __ldg(prow + f + 1);
  int cc[P];
  T cw[P];
#pragma unroll
  for (int q = 0; q < PN; ++q) {
    cc[q] = 0;
    cw[q] = T(0);
    if (k0 + q < k1) {
      cc[q] = __ldg(pcol + k0 + q);
      cw[q] = __ldg(pw + k0 + q);
    }
  }
  pdl_wait_then_trigger();
  T v[S];
#pragma unroll
  for (int r = 0; r < S; ++r) v[r] = T(0);
  if (sk != (1 << S) - 1) {
#pragma unroll
    for (int q = 0; q < PN; ++q)
      if (k0 + q < k1)
#pragma unroll
        for (int r = 0; r < S; ++r) v[r] = fma(cw[q] * dm.d[r], from[(size_t)cc[q] * S + r], v[r]);
    for (int k = k0 + PN; k < k1; ++k) {
      const int c = __ldg(pcol + k);
      const T w = __ldg(pw + k);
#pragma unroll
      for (int r = 0; r < S; ++r) v[r] = fma(w * dm.d[r], from[(size_t)c * S + r], v[r]);
    }
#pragma unroll
    for (int r = 0; r < S; ++r)
      if (sk & (1 << r)) v[r] = T(0);
  }
#pragma unroll
  for (int r = 0; r < S; ++r) {
    to[(size_t)f * S + r] = v[r];
    if (ACC) acc[(size_t)f * S + r] += v[r];
  }
}

// ------------------------------------------------------------ dnrm2x
// ugblas.cc:3156: per-component sums of squares over the NEW_DEFECT rows,
// accumulated in FP64 whatever the vector precision, in two deterministic
// stages (fixed grid, fixed reduction tree), then square roots.
// Both stages in one launch: every block writes its partial sums, takes a
// ticket, and the block that draws the last ticket adds the partials in
// block order (so the result does not depend on which block finishes last),
// writes the norms and resets the ticket counter for the next call.
template <class T, int S, bool ALL>
__global__ void __launch_bounds__(BLK) nrm_kernel(int n, const T *__restrict__ x, const uint8_t *__restrict__ flags,
                                                  double *__restrict__ partial, unsigned *__restrict__ ticket,
                                                  double *__restrict__ out) {
  pdl_prologue();
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!ALL && !(flags[i] & F_NEWDEF)) continue;
#pragma unroll
    for (int r = 0; r < S; ++r) {
      double v = double(x[(size_t)i * S + r]);
      acc[r] = fma(v, v, acc[r]);
    }
  }
  __shared__ double sh[BLK / 32][S];
  __shared__ bool last;
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < S) {
    double v = 0.0;
    for (int w = 0; w < BLK / 32; ++w) v += sh[w][threadIdx.x];
    partial[(size_t)blockIdx.x * S + threadIdx.x] = v;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ double red[BLK];
  for (int r = 0; r < S; ++r) {
    double v = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) v += __ldcg(partial + (size_t)b * S + r);
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[r] = sqrt(red[0]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

template <class T, int S, bool ALL>
__global__ void __launch_bounds__(BLK) nrm_stage1(int n, const T *__restrict__ x, const uint8_t *__restrict__ flags,
                                                  double *__restrict__ partial) {
  pdl_prologue();
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!ALL && !(flags[i] & F_NEWDEF)) continue;
#pragma unroll
    for (int r = 0; r < S; ++r) {
      double v = double(x[(size_t)i * S + r]);
      acc[r] = fma(v, v, acc[r]);
    }
  }
  __shared__ double sh[BLK / 32][S];
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < S) {
    double v = 0.0;
    for (int w = 0; w < BLK / 32; ++w) v += sh[w][threadIdx.x];
    partial[(size_t)blockIdx.x * S + threadIdx.x] = v;
  }
}

template <int S>
__global__ void nrm_stage2(int nblocks, const double *__restrict__ partial, double *__restrict__ out) {
  pdl_prologue();
  __shared__ double sh[1024];
  for (int r = 0; r < S; ++r) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v += partial[(size_t)b * S + r];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[r] = sqrt(sh[0]);
    __syncthreads();
  }
}

// ------------------------------------------------------------ cg (ls.cc:989-1064)
// ddot over the NEW_DEFECT rows (the surface of the top level), FP64, with the
// deterministic last-block reduction of nrm_kernel; the last block also does
// CGUpdate's scalar work on device scalars sc[], so a cg iteration needs no
// host round trip:
//   MODE 1: lambda = sum; f = lambda / rho; rho = lambda   (sc[CG_F], sc[CG_RHO])
//   MODE 2: lambda = sign * sum; alpha = rho / lambda, or a flag if lambda = 0
enum { CG_F = 0, CG_RHO = 1, CG_ALPHA = 2, CG_FLAG = 3 };
template <int MODE>
__device__ __forceinline__ void cg_scalars(double lam, double *sc) {
  if (MODE == 1) {
    sc[CG_F] = lam / sc[CG_RHO];
    sc[CG_RHO] = lam;
  } else if (lam == 0.0) {
    sc[CG_ALPHA] = 0.0;
    sc[CG_FLAG] = 1.0;
  } else {
    sc[CG_ALPHA] = sc[CG_RHO] / lam;
  }
}

template <int S, bool ALL, int MODE>
__global__ void __launch_bounds__(BLK) cg_dot_kernel(int n, const double *__restrict__ x, const double *__restrict__ y,
                                                     const uint8_t *__restrict__ flags, double *__restrict__ partial,
                                                     unsigned *__restrict__ ticket, double *__restrict__ sc,
                                                     double sign) {
  pdl_prologue();
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!ALL && !(flags[i] & F_NEWDEF)) continue;
#pragma unroll
    for (int r = 0; r < S; ++r) acc = fma(x[(size_t)i * S + r], y[(size_t)i * S + r], acc);
  }
  __shared__ double sh[BLK / 32];
  __shared__ bool last;
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < BLK / 32; ++w) v += sh[w];
    partial[blockIdx.x] = v;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ double red[BLK];
  double v = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) v += __ldcg(partial + b);
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    cg_scalars<MODE>(sign * red[0], sc);
    *ticket = 0u;
  }
}

// p = f p + c (dscal, then dadd: two roundings, as UG)
__global__ void cg_p_kernel(long long len, double *__restrict__ p, const double *__restrict__ c,
                            const double *__restrict__ sc) {
  pdl_prologue();
  const double f = sc[CG_F];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    p[i] = __dadd_rn(__dmul_rn(p[i], f), c[i]);
}

// x += alpha p; b -= alpha (A p), with tn = -(A p) (two daxpy, as UG)
__global__ void cg_xb_kernel(long long len, double *__restrict__ x, const double *__restrict__ p,
                             double *__restrict__ b, const double *__restrict__ tn, const double *__restrict__ sc) {
  pdl_prologue();
  const double a = sc[CG_ALPHA];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    x[i] = __dadd_rn(x[i], __dmul_rn(a, p[i]));
    b[i] = __dadd_rn(b[i], __dmul_rn(a, tn[i]));
  }
}

// b -= t (b += A c with t = -(A c))
__global__ void sub_kernel(long long len, double *__restrict__ b, const double *__restrict__ t) {
  pdl_prologue();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    b[i] = __dsub_rn(b[i], t[i]);
}

// ------------------------------------------------------------ bcgs (ls.cc:1864-2062)
// ddotw (ugblas.cc:3023, weights 1): per-component FP64 sums over the NEW_DEFECT
// rows, deterministic last-block reduction, then the components added in
// order; the last block also does the step's scalar work on sc[]:
//   RHO:   rho_new = d; beta = rho_new alpha / rho / omega if rho, omega != 0
//   ALPHA: a = sign d; alpha = a != 0 ? rho_new / a : a
//   TT:    tt = d
//   OMEGA: o = sign d; omega = tt != 0 ? o / tt : o; rho = rho_new
enum { BC_RHO = 0, BC_RHONEW = 1, BC_ALPHA = 2, BC_BETA = 3, BC_OMEGA = 4, BC_TT = 5, BC_HALF = 6 };
enum { BM_RHO = 0, BM_ALPHA = 1, BM_TT = 2, BM_OMEGA = 3 };
template <int MODE>
__device__ __forceinline__ void bcgs_scalars(double d, double sign, double *sc) {
  if (MODE == BM_RHO) {
    sc[BC_RHONEW] = d;
    if (sc[BC_RHO] != 0.0 && sc[BC_OMEGA] != 0.0) sc[BC_BETA] = d * sc[BC_ALPHA] / sc[BC_RHO] / sc[BC_OMEGA];
  } else if (MODE == BM_ALPHA) {
    const double a = sign * d;
    sc[BC_ALPHA] = a != 0.0 ? sc[BC_RHONEW] / a : a;
  } else if (MODE == BM_TT) {
    sc[BC_TT] = d;
  } else {
    const double o = sign * d;
    sc[BC_OMEGA] = sc[BC_TT] != 0.0 ? o / sc[BC_TT] : o;
    sc[BC_RHO] = sc[BC_RHONEW];
  }
}
template <int S, bool ALL, int MODE>
__global__ void __launch_bounds__(BLK) bcgs_dot_kernel(int n, const double *__restrict__ x, const double *__restrict__ y,
                                                       const uint8_t *__restrict__ flags, double *__restrict__ partial,
                                                       unsigned *__restrict__ ticket, double *__restrict__ sc,
                                                       double sign) {
  pdl_prologue();
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!ALL && !(flags[i] & F_NEWDEF)) continue;
#pragma unroll
    for (int r = 0; r < S; ++r) acc[r] = fma(x[(size_t)i * S + r], y[(size_t)i * S + r], acc[r]);
  }
  __shared__ double sh[BLK / 32][S];
  __shared__ bool last;
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < S) {
    double v = 0.0;
    for (int w = 0; w < BLK / 32; ++w) v += sh[w][threadIdx.x];
    partial[(size_t)blockIdx.x * S + threadIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ double red[S][BLK];
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) v += __ldcg(partial + (size_t)b * S + r);
    red[r][threadIdx.x] = v;
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int r = 0; r < S; ++r) red[r][threadIdx.x] += red[r][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double d = 0.0;
    for (int r = 0; r < S; ++r) d += 1.0 * red[r][0];
    bcgs_scalars<MODE>(d, sign, sc);
    *ticket = 0u;
  }
}

// p = beta p; p += b; p += (-beta omega) v, with vn = -v (three UG passes)
__global__ void bcgs_p_kernel(long long len, double *__restrict__ p, const double *__restrict__ b,
                              const double *__restrict__ vn, const double *__restrict__ sc) {
  pdl_prologue();
  const double beta = sc[BC_BETA], a = beta * sc[BC_OMEGA];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    p[i] = __dadd_rn(__dadd_rn(__dmul_rn(beta, p[i]), b[i]), __dmul_rn(a, vn[i]));
}

// x += alpha q; s = b; s += (-alpha) v, with vn = -v
__global__ void bcgs_xs_kernel(long long len, double *__restrict__ x, const double *__restrict__ q,
                               const double *__restrict__ b, double *__restrict__ sv, const double *__restrict__ vn,
                               const double *__restrict__ sc) {
  pdl_prologue();
  const double a = sc[BC_ALPHA];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    x[i] = __dadd_rn(x[i], __dmul_rn(a, q[i]));
    sv[i] = __dadd_rn(b[i], __dmul_rn(a, vn[i]));
  }
}

// the convergence test after the first half step, on the device: sc_cmp of
// the norms of s against abslimit or the reduction target (th[0..s), th[8..8+s))
__global__ void bcgs_half_test_kernel(int s, const double *__restrict__ norms, const double *__restrict__ th,
                                      double *__restrict__ sc) {
  pdl_prologue();
  if (threadIdx.x != 0) return;
  bool a = true, r = true;
  for (int k = 0; k < s; ++k) {
    if (fabs(norms[k]) >= fabs(th[k])) a = false;
    if (fabs(norms[k]) >= fabs(th[GMG_MAX_S + k])) r = false;
  }
  sc[BC_HALF] = (a || r) ? 1.0 : 0.0;
}

// second half: x += omega q; b = s; b += (-omega) t, with tn = -t -- or, when
// the first half already met the test, b = s (UG's break after dcopy(b, s))
__global__ void bcgs_xb_kernel(long long len, double *__restrict__ x, const double *__restrict__ q,
                               double *__restrict__ b, const double *__restrict__ sv, const double *__restrict__ tn,
                               const double *__restrict__ sc) {
  pdl_prologue();
  const bool half = sc[BC_HALF] != 0.0;
  const double o = sc[BC_OMEGA];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    if (half) {
      b[i] = sv[i];
    } else {
      x[i] = __dadd_rn(x[i], __dmul_rn(o, q[i]));
      b[i] = __dadd_rn(sv[i], __dmul_rn(o, tn[i]));
    }
  }
}

// ------------------------------------------------------------ batched ls
// The end of one ls iteration of a batched hierarchy, over the rows of every
// instance on its own finest level (all top levels in one launch):
//   SPMV (mixed precision):  b -= A c with the FP64 matrix (refinement defect);
//   LSUpdate:                x += c, unless the instance has converged (its x
//                            then stays that of its converged iteration);
//   dnrm2x:                  per-component norms of b on NEW_DEFECT rows.
// One block per chunk of one instance's rows (processing order); the block
// sums go to partial[], and the instance's last block to finish (a ticket
// per instance, reset by that block) adds them in chunk order, so the norms
// are deterministic.  c == nullptr: norms only.
struct FinishTop {
  const int *rows;
  const uint8_t *flags;
  const int *sptr, *scol;  // sliced ELLPACK (sptr == nullptr: block CSR below)
  const double *sval;
  const int *rowptr, *col;
  const double *val;
  void *b;
  double *x;
  const void *c;
};
struct FinishArgs {
  FinishTop t[GMG_MAX_TOPS];
};

template <class TB, class TC, int S, bool SPMV>
__global__ void __launch_bounds__(BLK) batch_finish_kernel(
    const __grid_constant__ FinishArgs A, const int *__restrict__ chunk_top, const int *__restrict__ chunk_id,
    const int *__restrict__ chunk_q0, const int *__restrict__ chunk_q1, const int *__restrict__ inst_c0,
    const int *__restrict__ inst_c1, const uint8_t *__restrict__ conv, double *__restrict__ partial,
    int *__restrict__ ticket, double *__restrict__ norms) {
  pdl_prologue();
  const int ch = blockIdx.x, id = chunk_id[ch], q0 = chunk_q0[ch], q1 = chunk_q1[ch];
  const FinishTop &T = A.t[chunk_top[ch]];
  TB *__restrict__ b = (TB *)T.b;
  const TC *__restrict__ c = (const TC *)T.c;
  double *__restrict__ x = T.x;
  const bool upd = c != nullptr && !conv[id];
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
    const int i = T.rows[q];
    TB bi[S];
#pragma unroll
    for (int r = 0; r < S; ++r) bi[r] = b[(size_t)i * S + r];
    if (SPMV) {
      double s[S];
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = 0.0;
      if (T.sptr) {  // sliced ELLPACK row i: entries sptr[i/32] + 32 k + i%32
        const int e0 = __ldg(T.sptr + (i >> 5));
        const int w = (__ldg(T.sptr + (i >> 5) + 1) - e0) >> 5;
        int e = e0 + (i & 31);
#pragma unroll 4
        for (int kk = 0; kk < w; ++kk, e += 32) {
          const int j = __ldg(T.scol + e);
          const double *m = T.sval + (size_t)e * (S * S);
#pragma unroll
          for (int cc = 0; cc < S; ++cc) {
            const double yv = double(c[(size_t)j * S + cc]);
#pragma unroll
            for (int r = 0; r < S; ++r) s[r] = fma(__ldg(m + r * S + cc), yv, s[r]);
          }
        }
      } else {
        for (int kk = __ldg(T.rowptr + i); kk < __ldg(T.rowptr + i + 1); ++kk) {
          const int j = __ldg(T.col + kk);
          const double *m = T.val + (size_t)kk * (S * S);
#pragma unroll
          for (int cc = 0; cc < S; ++cc) {
            const double yv = double(c[(size_t)j * S + cc]);
#pragma unroll
            for (int r = 0; r < S; ++r) s[r] = fma(__ldg(m + r * S + cc), yv, s[r]);
          }
        }
      }
#pragma unroll
      for (int r = 0; r < S; ++r) {
        bi[r] -= s[r];
        b[(size_t)i * S + r] = bi[r];
      }
    }
    if (upd)
#pragma unroll
      for (int r = 0; r < S; ++r) x[(size_t)i * S + r] += double(c[(size_t)i * S + r]);
    if (T.flags[i] & F_NEWDEF)
#pragma unroll
      for (int r = 0; r < S; ++r) {
        const double v = double(bi[r]);
        acc[r] = fma(v, v, acc[r]);
      }
  }
  __shared__ double sh[BLK / 32][S];
  __shared__ bool last;
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < S) {
    double v = 0.0;
    for (int w = 0; w < BLK / 32; ++w) v += sh[w][threadIdx.x];
    partial[(size_t)ch * S + threadIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket + id, 1) == inst_c1[id] - inst_c0[id] - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the instance's chunk sums: thread t adds chunks t, t+BLK, ... in order,
  // then a fixed-shape block reduction (deterministic for a given chunking)
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (int q = inst_c0[id] + threadIdx.x; q < inst_c1[id]; q += blockDim.x)
#pragma unroll
    for (int r = 0; r < S; ++r) acc[r] += __ldcg(partial + (size_t)q * S + r);
  __syncthreads();  // sh is reused
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < S) {
    double v = 0.0;
    for (int w = 0; w < BLK / 32; ++w) v += sh[w][threadIdx.x];
    norms[(size_t)id * GMG_MAX_S + threadIdx.x] = sqrt(v);
  }
  if (threadIdx.x == 0) ticket[id] = 0;
}

// element-wise passes over the top levels of a batched hierarchy in one launch
struct Segs {
  void *dst[GMG_MAX_TOPS];
  const void *src[GMG_MAX_TOPS];
  void *aux[GMG_MAX_TOPS];
  long long off[GMG_MAX_TOPS + 1];
  int n;
};

__device__ __forceinline__ int seg_of(const Segs &sg, long long g) {
  int t = 0;
  while (t + 1 < sg.n && g >= sg.off[t + 1]) ++t;
  return t;
}

// mixed-precision iteration start: b32 = b64 (dst <- src), c32 = 0 (aux)
__global__ void refine_prepare_multi_kernel(const __grid_constant__ Segs sg) {
  pdl_prologue();
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < sg.off[sg.n];
       g += (long long)gridDim.x * blockDim.x) {
    const int t = seg_of(sg, g);
    const long long i = g - sg.off[t];
    ((float *)sg.dst[t])[i] = float(((const double *)sg.src[t])[i]);
    ((float *)sg.aux[t])[i] = 0.0f;
  }
}

// c64 = c32
__global__ void widen_multi_kernel(const __grid_constant__ Segs sg) {
  pdl_prologue();
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < sg.off[sg.n];
       g += (long long)gridDim.x * blockDim.x) {
    const int t = seg_of(sg, g);
    const long long i = g - sg.off[t];
    ((double *)sg.dst[t])[i] = double(((const float *)sg.src[t])[i]);
  }
}

// ------------------------------------------------------------ base solver
// The lmgc base solver `ls $m 1 $I ex` (np/procs/ls.cc:637, iter.cc:8972):
// nothing happens when every component of |b| is below the base abslimit;
// otherwise t = A^{-1} b (the exact solve of the band LU, here an explicit
// FP64 inverse), b -= A t, c += t.  One CTA: the base level is tiny.
template <class T, int S>
__global__ void __launch_bounds__(1024) base_kernel(int n, const double *__restrict__ ainv, const int *__restrict__ rowptr,
                                                    const int *__restrict__ col, const T *__restrict__ val,
                                                    T *__restrict__ c, T *__restrict__ b, T *__restrict__ t,
                                                    Damp<double> abslimit) {
  pdl_prologue();
  __shared__ double red[S][32];
  __shared__ int skip;
  const int N = n * S;
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
#pragma unroll
    for (int r = 0; r < S; ++r) { double v = double(b[(size_t)i * S + r]); acc[r] += v * v; }
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) red[r][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int below = 1;
    for (int r = 0; r < S; ++r) {
      double v = 0.0;
      for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) v += red[r][w];
      if (fabs(sqrt(v)) >= fabs(abslimit.d[r])) below = 0;
    }
    skip = below;
  }
  __syncthreads();
  if (skip) return;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double v = 0.0;
    for (int j = 0; j < N; ++j) v = fma(ainv[(size_t)i * N + j], double(b[j]), v);
    t[i] = T(v);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    T s[S];
#pragma unroll
    for (int r = 0; r < S; ++r) s[r] = T(0);
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = col[k];
#pragma unroll
      for (int r = 0; r < S; ++r)
#pragma unroll
        for (int cc = 0; cc < S; ++cc) s[r] = fma(val[(size_t)k * S * S + r * S + cc], t[(size_t)j * S + cc], s[r]);
    }
#pragma unroll
    for (int r = 0; r < S; ++r) {
      b[(size_t)i * S + r] -= s[r];
      c[(size_t)i * S + r] += t[(size_t)i * S + r];
    }
  }
}

// The same on a block-diagonal level (a batched hierarchy's base level): one
// CTA per independent block, each with its own abslimit test and its own
// dense inverse, so every instance is solved exactly as if it were alone.
template <class T, int S>
__global__ void __launch_bounds__(256) base_block_kernel(const int *__restrict__ bptr, const int *__restrict__ brows,
                                                         const long long *__restrict__ aoff,
                                                         const double *__restrict__ ainv,
                                                         const int *__restrict__ rowptr, const int *__restrict__ col,
                                                         const T *__restrict__ val, T *__restrict__ c,
                                                         T *__restrict__ b, T *__restrict__ t, Damp<double> abslimit) {
  pdl_prologue();
  __shared__ double red[S][8];
  __shared__ int skip;
  const int r0 = bptr[blockIdx.x], m = bptr[blockIdx.x + 1] - r0, N = m * S;
  const int *rows = brows + r0;
  const double *A = ainv + aoff[blockIdx.x];
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (int q = threadIdx.x; q < m; q += blockDim.x)
#pragma unroll
    for (int r = 0; r < S; ++r) { double v = double(b[(size_t)rows[q] * S + r]); acc[r] += v * v; }
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) red[r][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int below = 1;
    for (int r = 0; r < S; ++r) {
      double v = 0.0;
      for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) v += red[r][w];
      if (fabs(sqrt(v)) >= fabs(abslimit.d[r])) below = 0;
    }
    skip = below;
  }
  __syncthreads();
  if (skip) return;
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    double v = 0.0;
    for (int j = 0; j < N; ++j) v = fma(A[(size_t)e * N + j], double(b[(size_t)rows[j / S] * S + j % S]), v);
    t[(size_t)rows[e / S] * S + e % S] = T(v);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < m; q += blockDim.x) {
    const int i = rows[q];
    T s[S];
#pragma unroll
    for (int r = 0; r < S; ++r) s[r] = T(0);
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = col[k];
#pragma unroll
      for (int r = 0; r < S; ++r)
#pragma unroll
        for (int cc = 0; cc < S; ++cc) s[r] = fma(val[(size_t)k * S * S + r * S + cc], t[(size_t)j * S + cc], s[r]);
    }
#pragma unroll
    for (int r = 0; r < S; ++r) {
      b[(size_t)i * S + r] -= s[r];
      c[(size_t)i * S + r] += t[(size_t)i * S + r];
    }
  }
}

// ------------------------------------------------------------ permutations
// packed instance vectors (instance-major, each in its own list order) <->
// the rows of one top level of a batched hierarchy
template <class T>
__global__ void pack_gather_kernel(T *dst, const double *__restrict__ src, const int *__restrict__ rows,
                                   const int *__restrict__ pack, int m, int s) {
  pdl_prologue();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  const int i = rows[q], p = pack[q];
  for (int r = 0; r < s; ++r) dst[(size_t)i * s + r] = T(src[(size_t)p * s + r]);
}
template <class T>
__global__ void pack_scatter_kernel(double *dst, const T *__restrict__ src, const int *__restrict__ rows,
                                    const int *__restrict__ pack, int m, int s) {
  pdl_prologue();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  const int i = rows[q], p = pack[q];
  for (int r = 0; r < s; ++r) dst[(size_t)p * s + r] = double(src[(size_t)i * s + r]);
}

template <class T>
__global__ void gather_kernel(T *dst, const double *__restrict__ src, const int *__restrict__ perm, int n, int s) {
  pdl_prologue();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p = perm[i];
  for (int r = 0; r < s; ++r) dst[(size_t)i * s + r] = T(src[(size_t)p * s + r]);
}
template <class T>
__global__ void scatter_kernel(double *dst, const T *__restrict__ src, const int *__restrict__ perm, int n, int s) {
  pdl_prologue();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p = perm[i];
  for (int r = 0; r < s; ++r) dst[(size_t)p * s + r] = double(src[(size_t)i * s + r]);
}

// ------------------------------------------------------------ dispatch helpers
#define LAUNCH_CHECK(mg)                                                         \
  do {                                                                           \
    (mg)->launches++;                                                            \
    cudaError_t e_ = cudaGetLastError();                                         \
    if (e_ != cudaSuccess) {                                                     \
      set_error("%s:%d kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      return 1;                                                                  \
    }                                                                            \
  } while (0)

inline int vec_grid(long long len) {
  long long g = (len + BLK - 1) / BLK;
  return int(g > 4 * 152 * 8 ? 4 * 152 * 8 : (g < 1 ? 1 : g));
}

template <class T, class TY, int S, bool ACC>
int spmv_dispatch_tpr(gmg_mg *mg, const Level &L, const T *val, T *x, const TY *y, TY *acc) {
  const int n = L.n;
  switch (L.tpr) {
#define CASE(TP)                                                                                           \
  case TP:                                                                                                 \
    if (use_prefetch(L, grid_for((long long)n * TP)))                                                      \
      GMG_LAUNCH((spmv_minus_kernel<T, TY, S, TP, ACC, 4>), grid_for((long long)n * TP), BLK, n, L.A.rowptr, \
                 L.A.col, val, y, x, acc);                                                                 \
    else                                                                                                   \
      GMG_LAUNCH((spmv_minus_kernel<T, TY, S, TP, ACC, 0>), grid_for((long long)n * TP), BLK, n, L.A.rowptr, \
                 L.A.col, val, y, x, acc);                                                                 \
    break;
    CASE(1) CASE(2) CASE(4) CASE(8) CASE(16) CASE(32)
#undef CASE
    default: set_error("bad threads-per-row %d", L.tpr); return 1;
  }
  LAUNCH_CHECK(mg);
  return 0;
}

template <class T>
const T *sell_val(const Level &L);
template <>
const double *sell_val<double>(const Level &L) { return L.sell_v64; }
template <>
const float *sell_val<float>(const Level &L) { return L.sell_v32; }
// bytes of a level's sliced-ELLPACK matrix stream in precision T
template <class T>
long long sell_bytes(const Level &L) { return L.sell_nent * ((long long)L.s * L.s * sizeof(T) + 4); }

template <class T, class TY, bool ACC>
int spmv_dispatch(gmg_mg *mg, const Level &L, const T *val, T *x, const TY *y, TY *acc) {
  if (L.sell && sell_val<T>(L)) {
    const T *sv = sell_val<T>(L);
    const bool pre = use_prefetch(L, grid_for(L.n));
    const bool st = use_stream(L, sell_bytes<T>(L));
#define SK(SS)                                                                                                   \
  if (pre)                                                                                                       \
    GMG_LAUNCH((sell_spmv_kernel<T, TY, TY, SS, ACC, PF<SS>::N>), grid_for(L.n), BLK, L.n, L.sell_ptr, L.sell_col, \
               sv, y, x, acc);                                                                                   \
  else if (st)                                                                                                   \
    GMG_LAUNCH((sell_spmv_kernel<T, TY, TY, SS, ACC, -1>), grid_for(L.n), BLK, L.n, L.sell_ptr, L.sell_col, sv, y, \
               x, acc);                                                                                          \
  else                                                                                                           \
    GMG_LAUNCH((sell_spmv_kernel<T, TY, TY, SS, ACC, 0>), grid_for(L.n), BLK, L.n, L.sell_ptr, L.sell_col, sv, y, \
               x, acc);
    switch (L.s) {
      case 1: SK(1) break;
      case 2: SK(2) break;
      case 3: SK(3) break;
      default: set_error("block size %d not compiled", L.s); return 1;
    }
#undef SK
    LAUNCH_CHECK(mg);
    return 0;
  }
  switch (L.s) {
    case 1: return spmv_dispatch_tpr<T, TY, 1, ACC>(mg, L, val, x, y, acc);
    case 2: return spmv_dispatch_tpr<T, TY, 2, ACC>(mg, L, val, x, y, acc);
    case 3: return spmv_dispatch_tpr<T, TY, 3, ACC>(mg, L, val, x, y, acc);
    default: set_error("block size %d not compiled", L.s); return 1;
  }
}

template <class T>
const T *mval(const DevCSR &M);
template <>
const double *mval<double>(const DevCSR &M) { return M.v64; }
template <>
const float *mval<float>(const DevCSR &M) { return M.v32; }
template <class T>
const T *dinv_of(const Level &L);
template <>
const double *dinv_of<double>(const Level &L) { return L.dinv64; }
template <>
const float *dinv_of<float>(const Level &L) { return L.dinv32; }
template <class T>
const T *udinv_of(const Level &L);
template <>
const double *udinv_of<double>(const Level &L) { return L.udinv64; }
template <>
const float *udinv_of<float>(const Level &L) { return L.udinv32; }

template <class T, int S, int TPR>
int gs_waves(gmg_mg *mg, const Level &L, T *t, const T *b) {
  const T *val = mval<T>(L.A), *dinv = dinv_of<T>(L);
  for (int w = 0; w < L.lower.nwave(); ++w) {
    const int r0 = L.lower.ptr[w], nr = L.lower.ptr[w + 1] - r0;
    if (nr <= 0) continue;
    const unsigned g = grid_for((long long)nr * TPR);
    const bool pre = g <= PREFETCH_MAX_BLOCKS;  // per wave (the autotuner times whole-level launches)
    if (L.all_active && pre)
      GMG_LAUNCH((gs_wave_kernel<T, S, TPR, true, 4>), g, BLK, L.lower.rows + r0, nr, L.A.rowptr, L.A.col, val, dinv,
                 L.flags, b, t);
    else if (L.all_active)
      GMG_LAUNCH((gs_wave_kernel<T, S, TPR, true, 0>), g, BLK, L.lower.rows + r0, nr, L.A.rowptr, L.A.col, val, dinv,
                 L.flags, b, t);
    else if (pre)
      GMG_LAUNCH((gs_wave_kernel<T, S, TPR, false, 4>), g, BLK, L.lower.rows + r0, nr, L.A.rowptr, L.A.col, val,
                 dinv, L.flags, b, t);
    else
      GMG_LAUNCH((gs_wave_kernel<T, S, TPR, false, 0>), g, BLK, L.lower.rows + r0, nr, L.A.rowptr, L.A.col, val,
                 dinv, L.flags, b, t);
    LAUNCH_CHECK(mg);
  }
  return 0;
}

// one cooperative launch of ilu_iface_kernel (grid: every block resident)
template <class T, int S, int TPR, bool ALL, bool FWD>
int iface_launch(gmg_mg *mg, const Level &L, const T *val, const T *dinv, T *t, const T *b) {
  auto kern = ilu_iface_kernel<T, S, TPR, ALL, FWD>;
  static thread_local std::map<void *, int> max_grid;
  int &mgrid = max_grid[(void *)kern];
  if (mgrid == 0) {
    int per_sm = 0, nsm = 0, dev = 0;
    GMG_CUDA(cudaGetDevice(&dev));
    GMG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    GMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BLK, 0));
    mgrid = std::max(1, per_sm * nsm);
  }
  const int nitems = FWD ? L.iface_fw_n : L.iface_bw_n;
  const long long need = ((long long)nitems * TPR + BLK - 1) / BLK;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(std::max<long long>(1, std::min<long long>(need, mgrid))));
  cfg.blockDim = dim3(BLK);
  cfg.stream = mg->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  const int nc = int(L.dom_cptr.size()) - 1;
  cudaLaunchKernelEx(&cfg, kern, (const int *)(FWD ? L.iface_fw_items : L.iface_bw_items), nitems, L.dom_nint,
                     L.dom_cptr[nc - 1], (const int *)(FWD ? L.L.rowptr : L.U.rowptr),
                     (const int *)(FWD ? L.L.col : L.U.col), val, dinv, (const uint8_t *)L.flags, b, t,
                     L.iface_flags + (FWD ? 0 : (L.n - L.dom_nint)), L.iface_ctr + (FWD ? 0 : 2), L.iface_err);
  LAUNCH_CHECK(mg);
  return 0;
}

// the ILU solve in subdomain order: interiors (one block per subdomain), the
// interface colours forward; the interface colours backward, interiors
template <class T, int S, int TPR, bool ALL>
int ilu_domain(gmg_mg *mg, const Level &L, T *t, const T *b) {
  const T *lv = mval<T>(L.L), *uv = mval<T>(L.U), *ud = udinv_of<T>(L);
  const int nc = int(L.dom_cptr.size()) - 1;
  const size_t fsm = region_smem_bytes<T, S>(L.dom_lt, true), bsm = region_smem_bytes<T, S>(L.dom_ut, false);
  const bool smem = L.dom_lt.ent0 && fsm <= 48 * 1024 && bsm <= 48 * 1024;
  if (smem)
    pdl_launch_smem(mg, ilu_region_smem_kernel<T, S, ALL, true>, dim3(L.dom_nreg), dim3(REGION_BLK), fsm,
                    L.dom_fwbeg, L.dom_fwptr, L.dom_frows, L.dom_lt.ent0, L.dom_lt.col, L.dom_lt.k, L.dom_lt.ext0,
                    L.dom_lt.ext, lv, (const T *)nullptr, L.flags, b, t, L.dom_lt.max_ent, L.dom_lt.max_rows);
  else
    GMG_LAUNCH((ilu_region_kernel<T, S, TPR, ALL, true>), L.dom_nreg, REGION_BLK, L.dom_fwbeg, L.dom_fwptr,
               L.dom_frows, L.L.rowptr, L.L.col, lv, (const T *)nullptr, L.flags, b, t);
  LAUNCH_CHECK(mg);
  if (L.iface_coop && (mg->iface_sweep == 2 || (mg->iface_sweep == 1 && sizeof(T) == 8))) {
    if (iface_launch<T, S, TPR, ALL, true>(mg, L, lv, ud, t, b) ||
        iface_launch<T, S, TPR, ALL, false>(mg, L, uv, ud, t, (const T *)nullptr))
      return 1;
  } else {
  // the last colour's rows have no upper entries: its forward and backward
  // steps are one launch
  for (int c = 0; c < nc; ++c) {
    const int r0 = L.dom_cptr[c], nr = L.dom_cptr[c + 1] - r0;
    if (nr <= 0) continue;
    if (c == nc - 1)
      GMG_LAUNCH((ilu_fwd_kernel<T, S, TPR, ALL, true>), grid_for((long long)nr * TPR), BLK,
                 L.dom_iface + (r0 - L.dom_nint), nr, L.L.rowptr, L.L.col, lv, L.flags, b, t, ud);
    else
      GMG_LAUNCH((ilu_fwd_kernel<T, S, TPR, ALL, false>), grid_for((long long)nr * TPR), BLK,
                 L.dom_iface + (r0 - L.dom_nint), nr, L.L.rowptr, L.L.col, lv, L.flags, b, t, (const T *)nullptr);
    LAUNCH_CHECK(mg);
  }
  for (int c = nc - 2; c >= 0; --c) {
    const int r0 = L.dom_cptr[c], nr = L.dom_cptr[c + 1] - r0;
    if (nr <= 0) continue;
    GMG_LAUNCH((ilu_bwd_kernel<T, S, TPR, ALL>), grid_for((long long)nr * TPR), BLK, L.dom_iface + (r0 - L.dom_nint),
               nr, L.U.rowptr, L.U.col, uv, ud, L.flags, t);
    LAUNCH_CHECK(mg);
  }
  }
  if (smem)
    pdl_launch_smem(mg, ilu_region_smem_kernel<T, S, ALL, false>, dim3(L.dom_nreg), dim3(REGION_BLK), bsm,
                    L.dom_bwbeg, L.dom_bwptr, L.dom_brows, L.dom_ut.ent0, L.dom_ut.col, L.dom_ut.k, L.dom_ut.ext0,
                    L.dom_ut.ext, uv, ud, L.flags, (const T *)nullptr, t, L.dom_ut.max_ent, L.dom_ut.max_rows);
  else
    GMG_LAUNCH((ilu_region_kernel<T, S, TPR, ALL, false>), L.dom_nreg, REGION_BLK, L.dom_bwbeg, L.dom_bwptr,
               L.dom_brows, L.U.rowptr, L.U.col, uv, ud, L.flags, (const T *)nullptr, t);
  LAUNCH_CHECK(mg);
  return 0;
}

template <class T, int S, int TPR>
int ilu_waves(gmg_mg *mg, const Level &L, T *t, const T *b) {
  if (L.dom_nreg > 0)
    return L.all_active ? ilu_domain<T, S, TPR, true>(mg, L, t, b) : ilu_domain<T, S, TPR, false>(mg, L, t, b);
  const T *lv = mval<T>(L.L), *uv = mval<T>(L.U), *ud = udinv_of<T>(L);
  for (int w = 0; w < L.lower.nwave(); ++w) {
    const int r0 = L.lower.ptr[w], nr = L.lower.ptr[w + 1] - r0;
    if (nr <= 0) continue;
    if (L.all_active)
      GMG_LAUNCH((ilu_fwd_kernel<T, S, TPR, true>), grid_for((long long)nr * TPR), BLK,
                 L.lower.rows + r0, nr, L.L.rowptr, L.L.col, lv, L.flags, b, t, (const T *)nullptr);
    else
      GMG_LAUNCH((ilu_fwd_kernel<T, S, TPR, false>), grid_for((long long)nr * TPR), BLK,
                 L.lower.rows + r0, nr, L.L.rowptr, L.L.col, lv, L.flags, b, t, (const T *)nullptr);
    LAUNCH_CHECK(mg);
  }
  for (int w = 0; w < L.upper.nwave(); ++w) {
    const int r0 = L.upper.ptr[w], nr = L.upper.ptr[w + 1] - r0;
    if (nr <= 0) continue;
    if (L.all_active)
      GMG_LAUNCH((ilu_bwd_kernel<T, S, TPR, true>), grid_for((long long)nr * TPR), BLK, 
          L.upper.rows + r0, nr, L.U.rowptr, L.U.col, uv, ud, L.flags, t);
    else
      GMG_LAUNCH((ilu_bwd_kernel<T, S, TPR, false>), grid_for((long long)nr * TPR), BLK, 
          L.upper.rows + r0, nr, L.U.rowptr, L.U.col, uv, ud, L.flags, t);
    LAUNCH_CHECK(mg);
  }
  return 0;
}

// threads per row for the triangular sweeps: short rows, so at most 8
inline int tri_tpr(const Level &L) { return L.tpr > 8 ? 8 : (L.tpr < 4 ? 4 : L.tpr); }

}  // namespace

// ============================================================ launchers
int k_set(gmg_mg *mg, int prec, void *x, long long len, double a) {
  if (len <= 0) return 0;
  if (prec == GMG_PREC_FP64) GMG_LAUNCH((set_kernel<double>), vec_grid(len), BLK, (double *)x, len, a);
  else GMG_LAUNCH((set_kernel<float>), vec_grid(len), BLK, (float *)x, len, float(a));
  LAUNCH_CHECK(mg);
  return 0;
}

int k_copy(gmg_mg *mg, int prec, void *x, const void *y, long long len) {
  if (len <= 0) return 0;
  if (prec == GMG_PREC_FP64) GMG_LAUNCH((copy_kernel<double>), vec_grid(len), BLK, (double *)x, (const double *)y, len);
  else GMG_LAUNCH((copy_kernel<float>), vec_grid(len), BLK, (float *)x, (const float *)y, len);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_add(gmg_mg *mg, int prec, void *x, const void *y, long long len) {
  if (len <= 0) return 0;
  if (prec == GMG_PREC_FP64) GMG_LAUNCH((add_kernel<double>), vec_grid(len), BLK, (double *)x, (const double *)y, len);
  else GMG_LAUNCH((add_kernel<float>), vec_grid(len), BLK, (float *)x, (const float *)y, len);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_scale(gmg_mg *mg, int prec, void *x, int n, int s, const double *damp) {
  bool unit = true;
  for (int r = 0; r < s; ++r) unit = unit && damp[r] == 1.0;
  if (unit || n <= 0) return 0;  // dscalx by 1 is the identity
#define SC(TT, SS) GMG_LAUNCH((scale_kernel<TT, SS>), grid_for(n), BLK, (TT *)x, n, make_damp<TT>(damp, SS))
  if (prec == GMG_PREC_FP64) {
    if (s == 1) SC(double, 1); else if (s == 2) SC(double, 2); else if (s == 3) SC(double, 3);
    else { set_error("block size %d not compiled", s); return 1; }
  } else {
    if (s == 1) SC(float, 1); else if (s == 2) SC(float, 2); else if (s == 3) SC(float, 3);
    else { set_error("block size %d not compiled", s); return 1; }
  }
#undef SC
  LAUNCH_CHECK(mg);
  return 0;
}

int k_convert(gmg_mg *mg, int dp, void *dst, int sp, const void *src, long long len) {
  if (len <= 0) return 0;
  if (dp == sp) return k_copy(mg, dp, dst, src, len);
  if (dp == GMG_PREC_FP32)
    GMG_LAUNCH((convert_kernel<float, double>), vec_grid(len), BLK, (float *)dst, (const double *)src, len);
  else
    GMG_LAUNCH((convert_kernel<double, float>), vec_grid(len), BLK, (double *)dst, (const float *)src, len);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_batch_finish(gmg_mg *mg, int bprec, gmg_vec *b, gmg_vec *x, int cprec, gmg_vec *c, bool spmv, int s) {
  const auto &B = mg->batch;
  if (B.nchunks_all == 0) return 0;
  GMG_CHECK(!spmv || (bprec == GMG_PREC_FP64 && c), "batched refinement update needs an FP64 defect and c");
  GMG_CHECK((int)B.tops.size() <= GMG_MAX_TOPS, "batched hierarchy with %zu top levels (at most %d)", B.tops.size(),
            GMG_MAX_TOPS);
  FinishArgs A{};
  for (size_t t = 0; t < B.tops.size(); ++t) {
    const int l = B.tops[t].level;
    const Level &L = mg->lev[l];
    FinishTop &T = A.t[t];
    T.rows = B.tops[t].rows_dev;
    T.flags = L.flags;
    T.sptr = L.sell ? L.sell_ptr : nullptr;
    T.scol = L.sell_col;
    T.sval = L.sell_v64;
    T.rowptr = L.A.rowptr;
    T.col = L.A.col;
    T.val = L.A.v64;
    T.b = b->lev[l];
    T.x = x ? (double *)x->lev[l] : nullptr;
    T.c = c ? c->lev[l] : nullptr;
  }
#define BF(TB, TC, SS, SP)                                                                                        \
  GMG_LAUNCH((batch_finish_kernel<TB, TC, SS, SP>), B.nchunks_all, BLK, A, B.chunk_top_dev, B.chunk_id_dev,       \
             B.chunk_q0_dev, B.chunk_q1_dev, B.inst_c0_dev, B.inst_c1_dev, B.conv_dev, B.partial_dev,             \
             B.ticket_dev, B.norms_dev)
#define BS(TB, TC, SP)                         \
  if (s == 1) BF(TB, TC, 1, SP);               \
  else if (s == 2) BF(TB, TC, 2, SP);          \
  else if (s == 3) BF(TB, TC, 3, SP);          \
  else { set_error("block size %d not compiled", s); return 1; }
  if (spmv) {
    if (cprec == GMG_PREC_FP32) { BS(double, float, true) } else { BS(double, double, true) }
  } else if (bprec == GMG_PREC_FP64) {
    if (cprec == GMG_PREC_FP64) { BS(double, double, false) } else { BS(double, float, false) }
  } else {
    if (cprec == GMG_PREC_FP64) { BS(float, double, false) } else { BS(float, float, false) }
  }
#undef BS
#undef BF
  LAUNCH_CHECK(mg);
  return 0;
}

static int top_segs(gmg_mg *mg, Segs &sg) {
  const auto &B = mg->batch;
  GMG_CHECK((int)B.tops.size() <= GMG_MAX_TOPS, "batched hierarchy with %zu top levels (at most %d)", B.tops.size(),
            GMG_MAX_TOPS);
  sg.n = int(B.tops.size());
  sg.off[0] = 0;
  for (int t = 0; t < sg.n; ++t) {
    const Level &L = mg->lev[B.tops[t].level];
    sg.off[t + 1] = sg.off[t] + (long long)L.n * L.s;
  }
  return 0;
}

int k_batch_refine_prepare(gmg_mg *mg, gmg_vec *b32, gmg_vec *c32, gmg_vec *b64) {
  Segs sg{};
  if (top_segs(mg, sg)) return 1;
  for (int t = 0; t < sg.n; ++t) {
    const int l = mg->batch.tops[t].level;
    sg.dst[t] = b32->lev[l];
    sg.src[t] = b64->lev[l];
    sg.aux[t] = c32->lev[l];
  }
  if (sg.off[sg.n] == 0) return 0;
  GMG_LAUNCH(refine_prepare_multi_kernel, vec_grid(sg.off[sg.n]), BLK, sg);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_batch_widen(gmg_mg *mg, gmg_vec *c64, gmg_vec *c32) {
  Segs sg{};
  if (top_segs(mg, sg)) return 1;
  for (int t = 0; t < sg.n; ++t) {
    const int l = mg->batch.tops[t].level;
    sg.dst[t] = c64->lev[l];
    sg.src[t] = c32->lev[l];
  }
  if (sg.off[sg.n] == 0) return 0;
  GMG_LAUNCH(widen_multi_kernel, vec_grid(sg.off[sg.n]), BLK, sg);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_refine_prepare(gmg_mg *mg, float *b32, float *c32, const double *b64, long long len) {
  if (len <= 0) return 0;
  GMG_LAUNCH(refine_prepare_kernel, vec_grid(len), BLK, b32, c32, b64, len);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_add_mixed(gmg_mg *mg, double *x, int sp, const void *c, long long len) {
  if (len <= 0) return 0;
  if (sp == GMG_PREC_FP64) return k_add(mg, GMG_PREC_FP64, x, c, len);
  GMG_LAUNCH((add_mixed_kernel<float>), vec_grid(len), BLK, x, (const float *)c, len);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_matmul_minus(gmg_mg *mg, const Level &L, int prec, void *x, const void *y, void *acc) {
  if (L.n == 0) return 0;
  if (prec == GMG_PREC_FP64) {
    if (acc) return spmv_dispatch<double, double, true>(mg, L, L.A.v64, (double *)x, (const double *)y, (double *)acc);
    return spmv_dispatch<double, double, false>(mg, L, L.A.v64, (double *)x, (const double *)y, nullptr);
  }
  GMG_CHECK(L.A.v32, "FP32 matrix copy not built (gmg_mg_opts.fp32_copy)");
  if (acc) return spmv_dispatch<float, float, true>(mg, L, L.A.v32, (float *)x, (const float *)y, (float *)acc);
  return spmv_dispatch<float, float, false>(mg, L, L.A.v32, (float *)x, (const float *)y, nullptr);
}

int k_matmul_minus_mixed(gmg_mg *mg, const Level &L, double *x, int yprec, const void *y) {
  if (yprec == GMG_PREC_FP64) return k_matmul_minus(mg, L, GMG_PREC_FP64, x, y, nullptr);
  return spmv_dispatch<double, float, false>(mg, L, L.A.v64, x, (const float *)y, nullptr);
}

int k_refine_update(gmg_mg *mg, const Level &L, double *b, double *x, const float *c) {
  if (L.n == 0) return 0;
  if (!L.sell) {  // small levels: two passes
    if (k_add_mixed(mg, x, GMG_PREC_FP32, c, (long long)L.n * L.s)) return 1;
    return k_matmul_minus_mixed(mg, L, b, GMG_PREC_FP32, c);
  }
  // the FP64 matrix is read once per ls iteration while the FP32 copies are
  // reused by every smoothing step of the cycle: above REFINE_STREAM_MIN_BYTES
  // it streams with evict-first loads so that it does not push them out of L2
  const bool st = sell_bytes<double>(L) > REFINE_STREAM_MIN_BYTES || use_stream(L, sell_bytes<double>(L));
  const bool pre = !st && use_prefetch(L, grid_for(L.n));
#define RU(SS)                                                                                                   \
  if (pre)                                                                                                       \
    GMG_LAUNCH((sell_spmv_kernel<double, float, double, SS, true, PF<SS>::N>), grid_for(L.n), BLK, L.n,          \
               L.sell_ptr, L.sell_col, L.sell_v64, c, b, x);                                                     \
  else if (st)                                                                                                   \
    GMG_LAUNCH((sell_spmv_kernel<double, float, double, SS, true, -1>), grid_for(L.n), BLK, L.n, L.sell_ptr,     \
               L.sell_col, L.sell_v64, c, b, x);                                                                 \
  else                                                                                                           \
    GMG_LAUNCH((sell_spmv_kernel<double, float, double, SS, true, 0>), grid_for(L.n), BLK, L.n, L.sell_ptr,      \
               L.sell_col, L.sell_v64, c, b, x);
  switch (L.s) {
    case 1: RU(1) break;
    case 2: RU(2) break;
    case 3: RU(3) break;
    default: set_error("block size %d not compiled", L.s); return 1;
  }
#undef RU
  LAUNCH_CHECK(mg);
  return 0;
}

int k_jac(gmg_mg *mg, const Level &L, int prec, void *t, const void *b, const double *damp) {
  if (L.n == 0) return 0;
#define JK(TT, SS, ALL)                                                                                     \
  GMG_LAUNCH((jac_kernel<TT, SS, ALL>), grid_for(L.n), BLK, L.n, dinv_of<TT>(L), L.flags, (const TT *)b, \
                                                                 (TT *)t, make_damp<TT>(damp, SS))
#define JS(TT)                                                                      \
  if (L.s == 1) { if (L.all_active) JK(TT, 1, true); else JK(TT, 1, false); }       \
  else if (L.s == 2) { if (L.all_active) JK(TT, 2, true); else JK(TT, 2, false); }  \
  else if (L.s == 3) { if (L.all_active) JK(TT, 3, true); else JK(TT, 3, false); }  \
  else { set_error("block size %d not compiled", L.s); return 1; }
  if (prec == GMG_PREC_FP64) { JS(double) }
  else { GMG_CHECK(L.dinv32, "FP32 copy not built"); JS(float) }
#undef JS
#undef JK
  LAUNCH_CHECK(mg);
  return 0;
}

template <class T, int S, bool ALL>
int jac_step_dispatch(gmg_mg *mg, const Level &L, T *bout, const T *bin, T *c, Damp<T> dm) {
  const T *dinv = dinv_of<T>(L);
  if (L.sell && sell_val<T>(L)) {
    if (use_prefetch(L, grid_for(L.n)))
      GMG_LAUNCH((sell_jac_step_kernel<T, S, ALL, PF<S>::N>), grid_for(L.n), BLK, L.n, L.sell_ptr, L.sell_col,
                 sell_val<T>(L), dinv, L.flags, bin, bout, c, dm);
    else if (use_stream(L, sell_bytes<T>(L)))
      GMG_LAUNCH((sell_jac_step_kernel<T, S, ALL, -1>), grid_for(L.n), BLK, L.n, L.sell_ptr, L.sell_col,
                 sell_val<T>(L), dinv, L.flags, bin, bout, c, dm);
    else
      GMG_LAUNCH((sell_jac_step_kernel<T, S, ALL, 0>), grid_for(L.n), BLK, L.n, L.sell_ptr, L.sell_col,
                 sell_val<T>(L), dinv, L.flags, bin, bout, c, dm);
    LAUNCH_CHECK(mg);
    return 0;
  }
  const T *val = mval<T>(L.A);
  switch (L.tpr) {
#define CASE(TP)                                                                                                 \
  case TP:                                                                                                       \
    GMG_LAUNCH((jac_step_kernel<T, S, TP, ALL>), grid_for((long long)L.n * TP), BLK, L.n, L.A.rowptr, L.A.col, val, \
               dinv, L.flags, bin, bout, c, dm);                                                                 \
    break;
    CASE(1) CASE(2) CASE(4) CASE(8) CASE(16) CASE(32)
#undef CASE
    default: set_error("bad threads-per-row %d", L.tpr); return 1;
  }
  LAUNCH_CHECK(mg);
  return 0;
}

int k_jac_step(gmg_mg *mg, const Level &L, int prec, void *bout, const void *bin, void *c, const double *damp) {
  if (L.n == 0) return 0;
#define JS(TT)                                                                                                  \
  {                                                                                                             \
    Damp<TT> dm = make_damp<TT>(damp, L.s);                                                                     \
    TT *o = (TT *)bout, *cc = (TT *)c;                                                                          \
    const TT *in = (const TT *)bin;                                                                             \
    if (L.s == 1) return L.all_active ? jac_step_dispatch<TT, 1, true>(mg, L, o, in, cc, dm)                    \
                                      : jac_step_dispatch<TT, 1, false>(mg, L, o, in, cc, dm);                  \
    if (L.s == 2) return L.all_active ? jac_step_dispatch<TT, 2, true>(mg, L, o, in, cc, dm)                    \
                                      : jac_step_dispatch<TT, 2, false>(mg, L, o, in, cc, dm);                  \
    if (L.s == 3) return L.all_active ? jac_step_dispatch<TT, 3, true>(mg, L, o, in, cc, dm)                    \
                                      : jac_step_dispatch<TT, 3, false>(mg, L, o, in, cc, dm);                  \
    set_error("block size %d not compiled", L.s);                                                               \
    return 1;                                                                                                   \
  }
  if (prec == GMG_PREC_FP64) JS(double)
  GMG_CHECK(L.dinv32 && L.A.v32, "FP32 copy not built");
  JS(float)
#undef JS
}

template <class T, int S>
int sell_gs_waves(gmg_mg *mg, const Level &L, T *t, const T *b) {
  const T *sv = sell_val<T>(L), *dinv = dinv_of<T>(L);
  const uint8_t *nl = L.sell_split ? L.sell_nl : nullptr;
  for (int w = 0; w < L.lower.nwave(); ++w) {
    const int r0 = L.lower.ptr[w], r1 = L.lower.ptr[w + 1];
    if (r1 <= r0) continue;
    const unsigned g = grid_for(r1 - r0);
    const bool pre = g <= PREFETCH_MAX_BLOCKS;  // per wave (the autotuner times whole-level launches)
    if (L.all_active && pre)
      GMG_LAUNCH((sell_gs_kernel<T, S, true, PF<S>::N>), g, BLK, r0, r1, L.sell_ptr, nl, L.sell_col, sv, dinv, L.flags,
                 b, t);
    else if (L.all_active)
      GMG_LAUNCH((sell_gs_kernel<T, S, true, 0>), g, BLK, r0, r1, L.sell_ptr, nl, L.sell_col, sv, dinv, L.flags, b, t);
    else if (pre)
      GMG_LAUNCH((sell_gs_kernel<T, S, false, PF<S>::N>), g, BLK, r0, r1, L.sell_ptr, nl, L.sell_col, sv, dinv, L.flags,
                 b, t);
    else
      GMG_LAUNCH((sell_gs_kernel<T, S, false, 0>), g, BLK, r0, r1, L.sell_ptr, nl, L.sell_col, sv, dinv, L.flags, b, t);
    LAUNCH_CHECK(mg);
  }
  return 0;
}

template <class T, int S>
int gs_chain(gmg_mg *mg, const Level &L, T *t, T *b, T *c, int steps, bool want_b) {
  const T *sv = sell_val<T>(L), *dinv = dinv_of<T>(L);
  const uint8_t *nl = L.sell_split ? L.sell_nl : nullptr;
  for (int st = 0; st < steps; ++st) {
    for (int w = 0; w < L.lower.nwave(); ++w) {
      const int r0 = L.lower.ptr[w], r1 = L.lower.ptr[w + 1];
      if (r1 <= r0) continue;
      const unsigned g = grid_for(r1 - r0);
      const bool pre = g <= PREFETCH_MAX_BLOCKS;  // per wave (the autotuner times whole-level launches)
      if (st == 0 && pre)
        GMG_LAUNCH((sell_gs_chain_kernel<T, S, true, PF<S>::N>), g, BLK, r0, r1, L.sell_ptr, nl, L.sell_col, sv, dinv, b,
                   t, c);
      else if (st == 0)
        GMG_LAUNCH((sell_gs_chain_kernel<T, S, true, 0>), g, BLK, r0, r1, L.sell_ptr, nl, L.sell_col, sv, dinv, b, t, c);
      else if (pre)
        GMG_LAUNCH((sell_gs_chain_kernel<T, S, false, PF<S>::N>), g, BLK, r0, r1, L.sell_ptr, nl, L.sell_col, sv, dinv, b,
                   t, c);
      else
        GMG_LAUNCH((sell_gs_chain_kernel<T, S, false, 0>), g, BLK, r0, r1, L.sell_ptr, nl, L.sell_col, sv, dinv, b, t,
                   c);
      LAUNCH_CHECK(mg);
    }
  }
  if (!want_b) return 0;
  const unsigned g = grid_for(L.n);
  if (use_prefetch(L, g))
    GMG_LAUNCH((sell_upper_defect_kernel<T, S, PF<S>::N>), g, BLK, L.n, L.sell_ptr, nl, L.sell_col, sv, t, b);
  else
    GMG_LAUNCH((sell_upper_defect_kernel<T, S, 0>), g, BLK, L.n, L.sell_ptr, nl, L.sell_col, sv, t, b);
  LAUNCH_CHECK(mg);
  return 0;
}

bool gs_chain_ok(const Level &L, int prec) {
  return L.sell && L.waves_contiguous && L.all_active && (prec == GMG_PREC_FP64 || (L.sell_v32 && L.dinv32));
}

long long gs_chain_cta_smem(const Level &L, int prec) {
  return 2ll * L.n * L.s * (prec == GMG_PREC_FP64 ? 8 : 4);
}

bool gs_chain_cta_ok(const Level &L, int prec) {
  return gs_chain_ok(L, prec) && L.lower.nwave() <= CTA_CHAIN_MAXW && gs_chain_cta_smem(L, prec) <= CTA_CHAIN_SMEM;
}

template <class T, int S>
static int gs_chain_cta(gmg_mg *mg, const Level &L, T *t, T *b, T *c, int steps, bool want_b) {
  constexpr int NT = S == 1 && sizeof(T) == 4 ? 1024 : 512;  // 64 / 128 registers a thread
  CtaWaves W{};
  W.n = L.n;
  W.nwave = L.lower.nwave();
  W.steps = steps;
  W.want_b = want_b;
  for (int w = 0; w <= W.nwave; ++w) W.ptr[w] = L.lower.ptr[w];
  const int smem = int(gs_chain_cta_smem(L, sizeof(T) == 8 ? GMG_PREC_FP64 : GMG_PREC_FP32));
  auto kern = sell_gs_chain_cta_kernel<T, S, PF<S>::N, NT>;
  static thread_local std::map<void *, int> smem_set;
  if (smem_set[(void *)kern] < smem) {
    GMG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    smem_set[(void *)kern] = smem;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(1);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = mg->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = mg->opts.disable_pdl ? 0 : 1;
  const uint8_t *nl = L.sell_split ? L.sell_nl : nullptr;
  cudaLaunchKernelEx(&cfg, kern, W, (const int *)L.sell_ptr, nl, (const int *)L.sell_col, sell_val<T>(L),
                     dinv_of<T>(L), b, t, c);
  LAUNCH_CHECK(mg);
  return 0;
}

template <class T, int S>
constexpr int cluster_chain_nt() {
  return S == 1 && sizeof(T) == 4 ? 1024 : 512;  // 64 / 128 registers a thread
}

// slots of the block of a cw-cluster with the most rows
static int cluster_chain_own(const Level &L, int cw) {
  int own = 0;
  for (int r = 0; r < cw; ++r) {
    int q = 0;
    for (int w = 0; w < L.lower.nwave(); ++w) q += cluster_share(L.lower.ptr[w + 1] - L.lower.ptr[w], cw, r);
    own = std::max(own, q);
  }
  return own;
}

// shared memory of the cluster form with the block's rows staged (rs) or streamed
static long long cluster_chain_bytes(const Level &L, int prec, int cw, bool rs) {
  const long long el = prec == GMG_PREC_FP64 ? 8 : 4, own = cluster_chain_own(L, cw), wm = std::max(L.sell_wmax - 1, 0);
  const long long s = L.s;
  return el * s * (L.n + own + own * s + (rs ? wm * own * s : 0)) +
         4 * ((rs ? wm * own : 0) + own + (rs ? 0 : own) + L.lower.nwave() + 1);
}

// 2: rows staged in shared memory, 1: rows streamed, 0: no cluster form
static int cluster_chain_form(const Level &L, int prec, int cw, int *smem) {
  if (!(cw == 2 || cw == 4 || cw == 8 || cw == 16)) return 0;
  if (!gs_chain_ok(L, prec) || L.lower.nwave() > CTA_CHAIN_MAXW) return 0;
  for (int rs = 1; rs >= 0; --rs) {
    const long long b = cluster_chain_bytes(L, prec, cw, rs != 0);
    if (b <= CLUSTER_CHAIN_SMEM) {
      *smem = int(b);
      return rs ? 2 : 1;
    }
  }
  return 0;
}

long long gs_chain_cluster_smem(const Level &L, int prec, int cw) {
  int smem = 0;
  return cluster_chain_form(L, prec, cw, &smem) ? smem : cluster_chain_bytes(L, prec, cw, false);
}

// the kernel with its launch attributes set for `smem` bytes; false where the
// device cannot co-schedule a cluster of cw such blocks (remembered)
template <class T, int S, bool RS>
static bool cluster_chain_prepare(int cw, int smem) {
  constexpr int NT = cluster_chain_nt<T, S>();
  auto kern = sell_gs_chain_cluster_kernel<T, S, PF<S>::N, NT, RS>;
  static std::mutex mu;
  static std::map<std::pair<int, int>, bool> fits;
  static int smem_set = 0, nonportable = 0;
  std::lock_guard<std::mutex> lk(mu);
  auto it = fits.find({cw, smem});
  if (it != fits.end()) return it->second;
  bool ok = true;
  if (smem_set < smem) {
    ok = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess;
    if (ok) smem_set = smem;
  }
  if (ok && cw > 8 && !nonportable) {
    ok = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
    if (ok) nonportable = 1;
  }
  if (ok) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cw);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cw;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    ok = cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters > 0;
  }
  cudaGetLastError();
  fits[{cw, smem}] = ok;
  return ok;
}

template <class T, int S>
static bool cluster_chain_prepare(int form, int cw, int smem) {
  return form == 2 ? cluster_chain_prepare<T, S, true>(cw, smem) : cluster_chain_prepare<T, S, false>(cw, smem);
}

bool gs_chain_cluster_ok(const Level &L, int prec, int cw) {
  int smem = 0;
  const int form = cluster_chain_form(L, prec, cw, &smem);
  if (!form) return false;
  if (prec == GMG_PREC_FP64) {
    if (L.s == 1) return cluster_chain_prepare<double, 1>(form, cw, smem);
    if (L.s == 2) return cluster_chain_prepare<double, 2>(form, cw, smem);
    if (L.s == 3) return cluster_chain_prepare<double, 3>(form, cw, smem);
  } else {
    if (L.s == 1) return cluster_chain_prepare<float, 1>(form, cw, smem);
    if (L.s == 2) return cluster_chain_prepare<float, 2>(form, cw, smem);
    if (L.s == 3) return cluster_chain_prepare<float, 3>(form, cw, smem);
  }
  return false;
}

template <class T, int S>
static int gs_chain_cluster(gmg_mg *mg, const Level &L, T *t, T *b, T *c, int steps, int cw, bool want_b) {
  constexpr int NT = cluster_chain_nt<T, S>();
  int smem = 0;
  const int form = cluster_chain_form(L, sizeof(T) == 8 ? GMG_PREC_FP64 : GMG_PREC_FP32, cw, &smem);
  GMG_CHECK(form, "no cluster form of %d blocks for this level", cw);
  CtaWaves W{};
  W.n = L.n;
  W.nwave = L.lower.nwave();
  W.steps = steps;
  W.own = cluster_chain_own(L, cw);
  W.want_b = want_b;
  W.wm = std::max(L.sell_wmax - 1, 0);
  for (int w = 0; w <= W.nwave; ++w) W.ptr[w] = L.lower.ptr[w];
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cw);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = mg->stream;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cw;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = mg->opts.disable_pdl ? 1 : 2;
  const uint8_t *nl = L.sell_split ? L.sell_nl : nullptr;
  if (form == 2)
    cudaLaunchKernelEx(&cfg, sell_gs_chain_cluster_kernel<T, S, PF<S>::N, NT, true>, W, (const int *)L.sell_ptr, nl,
                       (const int *)L.sell_col, sell_val<T>(L), dinv_of<T>(L), b, t, c);
  else
    cudaLaunchKernelEx(&cfg, sell_gs_chain_cluster_kernel<T, S, PF<S>::N, NT, false>, W, (const int *)L.sell_ptr, nl,
                       (const int *)L.sell_col, sell_val<T>(L), dinv_of<T>(L), b, t, c);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_gs_chain(gmg_mg *mg, const Level &L, int prec, void *t, void *b, void *c, int steps, bool want_b) {
  GMG_CHECK(gs_chain_ok(L, prec) && steps >= 1, "chained Gauss-Seidel steps need a colour-ordered SELL level");
  if (L.cta_chain > 1 && gs_chain_cluster_ok(L, prec, L.cta_chain)) {
    const int cw = L.cta_chain;
    if (prec == GMG_PREC_FP64) {
      if (L.s == 1) return gs_chain_cluster<double, 1>(mg, L, (double *)t, (double *)b, (double *)c, steps, cw, want_b);
      if (L.s == 2) return gs_chain_cluster<double, 2>(mg, L, (double *)t, (double *)b, (double *)c, steps, cw, want_b);
      if (L.s == 3) return gs_chain_cluster<double, 3>(mg, L, (double *)t, (double *)b, (double *)c, steps, cw, want_b);
    } else {
      if (L.s == 1) return gs_chain_cluster<float, 1>(mg, L, (float *)t, (float *)b, (float *)c, steps, cw, want_b);
      if (L.s == 2) return gs_chain_cluster<float, 2>(mg, L, (float *)t, (float *)b, (float *)c, steps, cw, want_b);
      if (L.s == 3) return gs_chain_cluster<float, 3>(mg, L, (float *)t, (float *)b, (float *)c, steps, cw, want_b);
    }
  }
  if (L.cta_chain == 1 && gs_chain_cta_ok(L, prec)) {
    if (prec == GMG_PREC_FP64) {
      if (L.s == 1) return gs_chain_cta<double, 1>(mg, L, (double *)t, (double *)b, (double *)c, steps, want_b);
      if (L.s == 2) return gs_chain_cta<double, 2>(mg, L, (double *)t, (double *)b, (double *)c, steps, want_b);
      if (L.s == 3) return gs_chain_cta<double, 3>(mg, L, (double *)t, (double *)b, (double *)c, steps, want_b);
    } else {
      if (L.s == 1) return gs_chain_cta<float, 1>(mg, L, (float *)t, (float *)b, (float *)c, steps, want_b);
      if (L.s == 2) return gs_chain_cta<float, 2>(mg, L, (float *)t, (float *)b, (float *)c, steps, want_b);
      if (L.s == 3) return gs_chain_cta<float, 3>(mg, L, (float *)t, (float *)b, (float *)c, steps, want_b);
    }
  }
  if (prec == GMG_PREC_FP64) {
    if (L.s == 1) return gs_chain<double, 1>(mg, L, (double *)t, (double *)b, (double *)c, steps, want_b);
    if (L.s == 2) return gs_chain<double, 2>(mg, L, (double *)t, (double *)b, (double *)c, steps, want_b);
    if (L.s == 3) return gs_chain<double, 3>(mg, L, (double *)t, (double *)b, (double *)c, steps, want_b);
  } else {
    if (L.s == 1) return gs_chain<float, 1>(mg, L, (float *)t, (float *)b, (float *)c, steps, want_b);
    if (L.s == 2) return gs_chain<float, 2>(mg, L, (float *)t, (float *)b, (float *)c, steps, want_b);
    if (L.s == 3) return gs_chain<float, 3>(mg, L, (float *)t, (float *)b, (float *)c, steps, want_b);
  }
  set_error("block size %d not compiled", L.s);
  return 1;
}

int k_gs(gmg_mg *mg, const Level &L, int prec, void *t, const void *b) {
  if (L.n == 0) return 0;
  if (L.sell && L.waves_contiguous) {
    if (prec == GMG_PREC_FP64) {
      if (L.s == 1) return sell_gs_waves<double, 1>(mg, L, (double *)t, (const double *)b);
      if (L.s == 2) return sell_gs_waves<double, 2>(mg, L, (double *)t, (const double *)b);
      if (L.s == 3) return sell_gs_waves<double, 3>(mg, L, (double *)t, (const double *)b);
    } else if (L.sell_v32 && L.dinv32) {
      if (L.s == 1) return sell_gs_waves<float, 1>(mg, L, (float *)t, (const float *)b);
      if (L.s == 2) return sell_gs_waves<float, 2>(mg, L, (float *)t, (const float *)b);
      if (L.s == 3) return sell_gs_waves<float, 3>(mg, L, (float *)t, (const float *)b);
    }
  }
  const int tp = tri_tpr(L);
#define GS(TT, SS)                                                                      \
  return tp == 4 ? gs_waves<TT, SS, 4>(mg, L, (TT *)t, (const TT *)b)                   \
                 : gs_waves<TT, SS, 8>(mg, L, (TT *)t, (const TT *)b);
  if (prec == GMG_PREC_FP64) {
    if (L.s == 1) { GS(double, 1) } else if (L.s == 2) { GS(double, 2) } else if (L.s == 3) { GS(double, 3) }
  } else {
    GMG_CHECK(L.A.v32 && L.dinv32, "FP32 copy not built");
    if (L.s == 1) { GS(float, 1) } else if (L.s == 2) { GS(float, 2) } else if (L.s == 3) { GS(float, 3) }
  }
#undef GS
  set_error("block size %d not compiled", L.s);
  return 1;
}

int k_luiter(gmg_mg *mg, const Level &L, int prec, void *t, const void *b) {
  if (L.n == 0) return 0;
  GMG_CHECK(L.ilu_ready, "ILU factors of level not computed (ilu PreProcess)");
  const int tp = tri_tpr(L);
#define IL(TT, SS)                                                                       \
  return tp == 4 ? ilu_waves<TT, SS, 4>(mg, L, (TT *)t, (const TT *)b)                   \
                 : ilu_waves<TT, SS, 8>(mg, L, (TT *)t, (const TT *)b);
  if (prec == GMG_PREC_FP64) {
    if (L.s == 1) { IL(double, 1) } else if (L.s == 2) { IL(double, 2) } else if (L.s == 3) { IL(double, 3) }
  } else {
    GMG_CHECK(L.L.v32, "FP32 ILU factors not built");
    if (L.s == 1) { IL(float, 1) } else if (L.s == 2) { IL(float, 2) } else if (L.s == 3) { IL(float, 3) }
  }
#undef IL
  set_error("block size %d not compiled", L.s);
  return 1;
}

// ------------------------------------------------------------ transfer by interpolation matrix
// RestrictByMatrix (transgrid.cc:1113-1247) as a gather over the transposed
// interpolation matrix (rows = coarse vectors, blocks coarse-component major):
// reset rows (VNCLASS >= NEWDEF) start from zero, the others keep their value;
// each block adds M d_v in the components the coarse VECSKIP leaves free; the
// reset rows are then scaled by damp (if any damp != 1, SCALE).  zc (optional)
// is set to zero on the coarse level in the same pass.
template <class T, int S, bool SCALE>
__global__ void __launch_bounds__(BLK) restrict_imat_kernel(int nc, const int *__restrict__ rrow,
                                                            const int *__restrict__ rcol, const T *__restrict__ rval,
                                                            const uint8_t *__restrict__ cflags,
                                                            const uint8_t *__restrict__ cskip,
                                                            const T *__restrict__ from, T *__restrict__ to, Damp<T> dm,
                                                            T *__restrict__ zc) {
  pdl_prologue();
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nc) return;
  const bool reset = __ldg(cflags + w) & F_RESET;
  const int sk = __ldg(cskip + w);
  T acc[S];
#pragma unroll
  for (int i = 0; i < S; ++i) acc[i] = reset ? T(0) : to[(size_t)w * S + i];
  for (int k = __ldg(rrow + w); k < __ldg(rrow + w + 1); ++k) {
    const int v = __ldg(rcol + k);
    const T *m = rval + (size_t)k * S * S;
    T d[S];
#pragma unroll
    for (int j = 0; j < S; ++j) d[j] = from[(size_t)v * S + j];
#pragma unroll
    for (int i = 0; i < S; ++i) {
      if (sk & (1 << i)) continue;
      T sum = T(0);
#pragma unroll
      for (int j = 0; j < S; ++j) sum = fma(__ldg(m + i * S + j), d[j], sum);
      acc[i] += sum;
    }
  }
#pragma unroll
  for (int i = 0; i < S; ++i) {
    to[(size_t)w * S + i] = (SCALE && reset) ? acc[i] * dm.d[i] : acc[i];
    if (zc) zc[(size_t)w * S + i] = T(0);
  }
}

// InterpolateCorrectionByMatrix (transgrid.cc:1292-1386): every fine vector
// takes the transposed blocks of its interpolation matrix times the coarse
// vectors in the components its VECSKIP leaves free (0 in the others), times
// damp; ACC: acc += t as well (lmgc's dadd(c, t))
template <class T, int S, bool ACC>
__global__ void __launch_bounds__(BLK) interp_imat_kernel(int nf, const int *__restrict__ prow,
                                                          const int *__restrict__ pcol, const T *__restrict__ pval,
                                                          const uint8_t *__restrict__ fskip,
                                                          const T *__restrict__ from, T *__restrict__ to, Damp<T> dm,
                                                          T *__restrict__ acc) {
  pdl_prologue();
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nf) return;
  const int sk = __ldg(fskip + v);
  T t[S];
#pragma unroll
  for (int i = 0; i < S; ++i) t[i] = T(0);
  for (int k = __ldg(prow + v); k < __ldg(prow + v + 1); ++k) {
    const int w = __ldg(pcol + k);
    const T *m = pval + (size_t)k * S * S;
    T c[S];
#pragma unroll
    for (int j = 0; j < S; ++j) c[j] = from[(size_t)w * S + j];
#pragma unroll
    for (int i = 0; i < S; ++i) {
      T sum = T(0);
#pragma unroll
      for (int j = 0; j < S; ++j) sum = fma(__ldg(m + j * S + i), c[j], sum);
      t[i] += sum;
    }
  }
#pragma unroll
  for (int i = 0; i < S; ++i) {
    const T r = (sk & (1 << i)) ? T(0) : t[i] * dm.d[i];
    to[(size_t)v * S + i] = r;
    if (ACC) acc[(size_t)v * S + i] += r;
  }
}

int k_restrict_imat(gmg_mg *mg, const Level &F, const Level &C, int prec, void *to, const void *from,
                    const double *damp, void *zero_coarse) {
  GMG_CHECK(F.has_imat, "RestrictByMatrix: no interpolation matrix on this level");
  if (C.n == 0) return 0;
  bool scale = false;
  for (int r = 0; r < F.s; ++r) scale = scale || damp[r] != 1.0;
#define RM(TT, SS)                                                                                            \
  do {                                                                                                        \
    if (scale)                                                                                                \
      GMG_LAUNCH((restrict_imat_kernel<TT, SS, true>), grid_for(C.n), BLK, C.n, F.IR.rowptr, F.IR.col,       \
                 mval<TT>(F.IR), C.flags, C.skip, (const TT *)from, (TT *)to, make_damp<TT>(damp, SS),        \
                 (TT *)zero_coarse);                                                                          \
    else                                                                                                      \
      GMG_LAUNCH((restrict_imat_kernel<TT, SS, false>), grid_for(C.n), BLK, C.n, F.IR.rowptr, F.IR.col,      \
                 mval<TT>(F.IR), C.flags, C.skip, (const TT *)from, (TT *)to, make_damp<TT>(damp, SS),        \
                 (TT *)zero_coarse);                                                                          \
  } while (0)
#define RMS(TT)                                 \
  if (F.s == 1) RM(TT, 1);                      \
  else if (F.s == 2) RM(TT, 2);                 \
  else if (F.s == 3) RM(TT, 3);                 \
  else { set_error("block size %d not compiled", F.s); return 1; }
  if (prec == GMG_PREC_FP64) { RMS(double) }
  else { GMG_CHECK(F.IR.v32, "FP32 interpolation matrix not built"); RMS(float) }
#undef RMS
#undef RM
  LAUNCH_CHECK(mg);
  return 0;
}

int k_interpolate_imat(gmg_mg *mg, const Level &F, int prec, void *to, const void *from, const double *damp,
                       void *acc) {
  GMG_CHECK(F.has_imat, "InterpolateCorrectionByMatrix: no interpolation matrix on this level");
  if (F.n == 0) return 0;
#define IM(TT, SS)                                                                                             \
  do {                                                                                                         \
    if (acc)                                                                                                   \
      GMG_LAUNCH((interp_imat_kernel<TT, SS, true>), grid_for(F.n), BLK, F.n, F.IP.rowptr, F.IP.col,          \
                 mval<TT>(F.IP), F.skip, (const TT *)from, (TT *)to, make_damp<TT>(damp, SS), (TT *)acc);      \
    else                                                                                                       \
      GMG_LAUNCH((interp_imat_kernel<TT, SS, false>), grid_for(F.n), BLK, F.n, F.IP.rowptr, F.IP.col,         \
                 mval<TT>(F.IP), F.skip, (const TT *)from, (TT *)to, make_damp<TT>(damp, SS), (TT *)acc);      \
  } while (0)
#define IMS(TT)                                 \
  if (F.s == 1) IM(TT, 1);                      \
  else if (F.s == 2) IM(TT, 2);                 \
  else if (F.s == 3) IM(TT, 3);                 \
  else { set_error("block size %d not compiled", F.s); return 1; }
  if (prec == GMG_PREC_FP64) { IMS(double) }
  else { GMG_CHECK(F.IP.v32, "FP32 interpolation matrix not built"); IMS(float) }
#undef IMS
#undef IM
  LAUNCH_CHECK(mg);
  return 0;
}

int k_restrict(gmg_mg *mg, const Level &F, const Level &C, int prec, void *to, const void *from, const double *damp,
               void *zero_coarse) {
  if (C.n == 0) return 0;
  const bool pre = use_prefetch(C, grid_for(C.n));
#define RK(TT, SS)                                                                                                 \
  do {                                                                                                             \
    if (pre)                                                                                                       \
      GMG_LAUNCH((restrict_kernel<TT, SS, 16>), grid_for(C.n), BLK, C.n, F.R.rowptr, F.R.col, mval<TT>(F.R),     \
                 C.flags, C.skip, (const TT *)from, (TT *)to, make_damp<TT>(damp, SS), (TT *)zero_coarse);         \
    else                                                                                                           \
      GMG_LAUNCH((restrict_kernel<TT, SS, 0>), grid_for(C.n), BLK, C.n, F.R.rowptr, F.R.col, mval<TT>(F.R),      \
                 C.flags, C.skip, (const TT *)from, (TT *)to, make_damp<TT>(damp, SS), (TT *)zero_coarse);         \
  } while (0)
#define RS(TT)                                  \
  if (F.s == 1) RK(TT, 1);                      \
  else if (F.s == 2) RK(TT, 2);                 \
  else if (F.s == 3) RK(TT, 3);                 \
  else { set_error("block size %d not compiled", F.s); return 1; }
  if (prec == GMG_PREC_FP64) { RS(double) }
  else { GMG_CHECK(F.R.v32, "FP32 transfer not built"); RS(float) }
#undef RS
#undef RK
  LAUNCH_CHECK(mg);
  return 0;
}

int k_interpolate(gmg_mg *mg, const Level &F, int prec, void *to, const void *from, const double *damp, void *acc) {
  if (F.n == 0) return 0;
  const bool pre = use_prefetch(F, grid_for(F.n));
#define IK(TT, SS, A)                                                                                              \
  do {                                                                                                             \
    if (pre)                                                                                                       \
      GMG_LAUNCH((interp_kernel<TT, SS, A, 4>), grid_for(F.n), BLK, F.n, F.P.rowptr, F.P.col, mval<TT>(F.P),      \
                 F.skip, (const TT *)from, (TT *)to, make_damp<TT>(damp, SS), (TT *)acc);                          \
    else                                                                                                           \
      GMG_LAUNCH((interp_kernel<TT, SS, A, 0>), grid_for(F.n), BLK, F.n, F.P.rowptr, F.P.col, mval<TT>(F.P),      \
                 F.skip, (const TT *)from, (TT *)to, make_damp<TT>(damp, SS), (TT *)acc);                          \
  } while (0)
#define IS(TT)                                                                \
  if (F.s == 1) { if (acc) IK(TT, 1, true); else IK(TT, 1, false); }         \
  else if (F.s == 2) { if (acc) IK(TT, 2, true); else IK(TT, 2, false); }    \
  else if (F.s == 3) { if (acc) IK(TT, 3, true); else IK(TT, 3, false); }    \
  else { set_error("block size %d not compiled", F.s); return 1; }
  if (prec == GMG_PREC_FP64) { IS(double) }
  else { GMG_CHECK(F.P.v32, "FP32 transfer not built"); IS(float) }
#undef IS
#undef IK
  LAUNCH_CHECK(mg);
  return 0;
}

int k_nrm2x(gmg_mg *mg, const Level &L, int prec, const void *x) {
  const int nb = REDUCE_BLOCKS;
  bool all = L.all_active;  // every row ACTIVE implies every row NEW_DEFECT
  unsigned *ticket = reinterpret_cast<unsigned *>(mg->norms_dev + GMG_MAX_S);
#define N1(TT, SS)                                                                                                  \
  { if (all) GMG_LAUNCH((nrm_kernel<TT, SS, true>), nb, BLK, L.n, (const TT *)x, L.flags, mg->partial, ticket,      \
                        mg->norms_dev);                                                                             \
    else GMG_LAUNCH((nrm_kernel<TT, SS, false>), nb, BLK, L.n, (const TT *)x, L.flags, mg->partial, ticket,         \
                    mg->norms_dev);                                                                                 \
    LAUNCH_CHECK(mg); return 0; }
  if (prec == GMG_PREC_FP64) {
    if (L.s == 1) N1(double, 1) if (L.s == 2) N1(double, 2) if (L.s == 3) N1(double, 3)
  } else {
    if (L.s == 1) N1(float, 1) if (L.s == 2) N1(float, 2) if (L.s == 3) N1(float, 3)
  }
#undef N1
  set_error("block size %d not compiled", L.s);
  return 1;
}

int k_cg_dot(gmg_mg *mg, const Level &L, const double *x, const double *y, double *sc, int mode, double sign) {
  unsigned *ticket = reinterpret_cast<unsigned *>(mg->norms_dev + GMG_MAX_S);
  const bool all = L.all_active;
#define CD(SS, A, M) GMG_LAUNCH((cg_dot_kernel<SS, A, M>), REDUCE_BLOCKS, BLK, L.n, x, y, L.flags, mg->partial, ticket, sc, sign)
#define CM(SS)                                                   \
  if (mode == 1) { if (all) CD(SS, true, 1); else CD(SS, false, 1); } \
  else { if (all) CD(SS, true, 2); else CD(SS, false, 2); }
  if (L.s == 1) { CM(1) } else if (L.s == 2) { CM(2) } else if (L.s == 3) { CM(3) }
  else { set_error("block size %d not compiled", L.s); return 1; }
#undef CM
#undef CD
  LAUNCH_CHECK(mg);
  return 0;
}

int k_cg_p(gmg_mg *mg, long long len, double *p, const double *c, const double *sc) {
  GMG_LAUNCH(cg_p_kernel, vec_grid(len), BLK, len, p, c, sc);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_cg_xb(gmg_mg *mg, long long len, double *x, const double *p, double *b, const double *tn, const double *sc) {
  GMG_LAUNCH(cg_xb_kernel, vec_grid(len), BLK, len, x, p, b, tn, sc);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_sub(gmg_mg *mg, long long len, double *b, const double *t) {
  GMG_LAUNCH(sub_kernel, vec_grid(len), BLK, len, b, t);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_bcgs_dot(gmg_mg *mg, const Level &L, const double *x, const double *y, double *sc, int mode, double sign) {
  unsigned *ticket = reinterpret_cast<unsigned *>(mg->norms_dev + GMG_MAX_S);
  const bool all = L.all_active;
#define BD(SS, A, M) GMG_LAUNCH((bcgs_dot_kernel<SS, A, M>), REDUCE_BLOCKS, BLK, L.n, x, y, L.flags, mg->partial, ticket, sc, sign)
#define BM(SS, A)                                                                        \
  switch (mode) {                                                                        \
    case 0: BD(SS, A, 0); break;                                                         \
    case 1: BD(SS, A, 1); break;                                                         \
    case 2: BD(SS, A, 2); break;                                                         \
    default: BD(SS, A, 3); break;                                                        \
  }
#define BA(SS) if (all) { BM(SS, true) } else { BM(SS, false) }
  if (L.s == 1) { BA(1) } else if (L.s == 2) { BA(2) } else if (L.s == 3) { BA(3) }
  else { set_error("block size %d not compiled", L.s); return 1; }
#undef BA
#undef BM
#undef BD
  LAUNCH_CHECK(mg);
  return 0;
}

int k_bcgs_p(gmg_mg *mg, long long len, double *p, const double *b, const double *vn, const double *sc) {
  GMG_LAUNCH(bcgs_p_kernel, vec_grid(len), BLK, len, p, b, vn, sc);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_bcgs_xs(gmg_mg *mg, long long len, double *x, const double *q, const double *b, double *sv, const double *vn,
              const double *sc) {
  GMG_LAUNCH(bcgs_xs_kernel, vec_grid(len), BLK, len, x, q, b, sv, vn, sc);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_bcgs_half_test(gmg_mg *mg, int s, const double *th, double *sc) {
  GMG_LAUNCH(bcgs_half_test_kernel, 1, 32, s, mg->norms_dev, th, sc);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_bcgs_xb(gmg_mg *mg, long long len, double *x, const double *q, double *b, const double *sv, const double *tn,
              const double *sc) {
  GMG_LAUNCH(bcgs_xb_kernel, vec_grid(len), BLK, len, x, q, b, sv, tn, sc);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_base_solve(gmg_mg *mg, const Level &L, int prec, void *c, void *b, void *t, const double *abslimit) {
  GMG_CHECK(L.ainv, "base level inverse not computed (ex PreProcess)");
  Damp<double> al = make_damp<double>(abslimit, L.s);
#define BK(TT, SS)                                                                                             \
  do {                                                                                                         \
    if (L.nblk_dev > 0)                                                                                        \
      GMG_LAUNCH((base_block_kernel<TT, SS>), L.nblk_dev, 256, L.blk_ptr_dev, L.blk_rows_dev, L.blk_aoff_dev,  \
                 L.ainv, L.A.rowptr, L.A.col, mval<TT>(L.A), (TT *)c, (TT *)b, (TT *)t, al);                   \
    else                                                                                                       \
      GMG_LAUNCH((base_kernel<TT, SS>), 1, 1024, L.n, L.ainv, L.A.rowptr, L.A.col, mval<TT>(L.A), (TT *)c,     \
                 (TT *)b, (TT *)t, al);                                                                        \
  } while (0)
#define BS(TT)                                   \
  if (L.s == 1) BK(TT, 1);                       \
  else if (L.s == 2) BK(TT, 2);                  \
  else if (L.s == 3) BK(TT, 3);                  \
  else { set_error("block size %d not compiled", L.s); return 1; }
  if (prec == GMG_PREC_FP64) { BS(double) }
  else { GMG_CHECK(L.A.v32, "FP32 copy not built"); BS(float) }
#undef BS
#undef BK
  LAUNCH_CHECK(mg);
  return 0;
}

int k_pack_gather(gmg_mg *mg, int prec, void *dst, const double *packed, const gmg_mg::Batch::TopLevel &tl, int s) {
  if (tl.nrows == 0) return 0;
  if (prec == GMG_PREC_FP64)
    GMG_LAUNCH((pack_gather_kernel<double>), grid_for(tl.nrows), BLK, (double *)dst, packed, tl.rows_dev,
               tl.pack_dev, tl.nrows, s);
  else
    GMG_LAUNCH((pack_gather_kernel<float>), grid_for(tl.nrows), BLK, (float *)dst, packed, tl.rows_dev,
               tl.pack_dev, tl.nrows, s);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_pack_scatter(gmg_mg *mg, int prec, double *packed, const void *src, const gmg_mg::Batch::TopLevel &tl, int s) {
  if (tl.nrows == 0) return 0;
  if (prec == GMG_PREC_FP64)
    GMG_LAUNCH((pack_scatter_kernel<double>), grid_for(tl.nrows), BLK, packed, (const double *)src, tl.rows_dev,
               tl.pack_dev, tl.nrows, s);
  else
    GMG_LAUNCH((pack_scatter_kernel<float>), grid_for(tl.nrows), BLK, packed, (const float *)src, tl.rows_dev,
               tl.pack_dev, tl.nrows, s);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_pack_scatter_range(gmg_mg *mg, int prec, double *packed, const void *src, const int *rows, const int *pack, int m,
                         int s) {
  if (m == 0) return 0;
  if (prec == GMG_PREC_FP64)
    GMG_LAUNCH((pack_scatter_kernel<double>), grid_for(m), BLK, packed, (const double *)src, rows, pack, m, s);
  else
    GMG_LAUNCH((pack_scatter_kernel<float>), grid_for(m), BLK, packed, (const float *)src, rows, pack, m, s);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_gather(gmg_mg *mg, int prec, void *dst, const double *src, const int *perm, int n, int s) {
  if (n == 0) return 0;
  if (prec == GMG_PREC_FP64) GMG_LAUNCH((gather_kernel<double>), grid_for(n), BLK, (double *)dst, src, perm, n, s);
  else GMG_LAUNCH((gather_kernel<float>), grid_for(n), BLK, (float *)dst, src, perm, n, s);
  LAUNCH_CHECK(mg);
  return 0;
}

int k_scatter(gmg_mg *mg, int prec, double *dst, const void *src, const int *perm, int n, int s) {
  if (n == 0) return 0;
  if (prec == GMG_PREC_FP64) GMG_LAUNCH((scatter_kernel<double>), grid_for(n), BLK, dst, (const double *)src, perm, n, s);
  else GMG_LAUNCH((scatter_kernel<float>), grid_for(n), BLK, dst, (const float *)src, perm, n, s);
  LAUNCH_CHECK(mg);
  return 0;
}

// the test of ls's loop after one device-side iteration: the same
// comparisons as the host loop (sc_cmp, npscan.cc:1027: every |d_r| < |lim_r|)
__global__ void ls_loop_test_kernel(LsLoopState *st, const double *__restrict__ norms, const double *flag,
                                    cudaGraphConditionalHandle h) {
  if (threadIdx.x != 0) return;
  const int it = st->it + 1, s = st->s;
  st->it = it;
  if (flag && *flag != 0.0) {
    st->flagged = it;
    cudaGraphSetConditional(h, 0);
    return;
  }
  bool finite = true, below_abs = true, below_reach = true;
  for (int r = 0; r < s; ++r) {
    const double d = norms[r];
    st->last[r] = d;
    finite = finite && isfinite(d);
    below_abs = below_abs && fabs(d) < fabs(st->abs[r]);
    below_reach = below_reach && fabs(d) < fabs(st->reach[r]);
  }
  if (!finite) {
    st->bad = it;
    cudaGraphSetConditional(h, 0);
    return;
  }
  if (below_abs || below_reach) st->conv = 1;
  cudaGraphSetConditional(h, (!st->conv && it < st->maxit) ? 1u : 0u);
}

int k_ls_loop_test(gmg_mg *mg, LsLoopState *st, const double *flag, cudaGraphConditionalHandle h) {
  ls_loop_test_kernel<<<1, 32, 0, mg->stream>>>(st, mg->norms_dev, flag, h);
  LAUNCH_CHECK(mg);
  return 0;
}

// the per-instance test of the batched ls loop (the host loop's comparisons,
// instance by instance); one block
__global__ void __launch_bounds__(1024) batch_loop_test_kernel(BatchLoopHead *hd, const double *__restrict__ norms,
                                                               uint8_t *conv, int *iters, double *last,
                                                               const double *__restrict__ reach,
                                                               cudaGraphConditionalHandle h) {
  const int it = hd->it + 1, ni = hd->ninst, s = hd->s;
  int all = 1;
  for (int k = threadIdx.x; k < ni; k += blockDim.x) {
    if (conv[k]) continue;
    const double *d = norms + (size_t)k * GMG_MAX_S;
    bool finite = true, below_abs = true, below_reach = true;
    for (int r = 0; r < s; ++r) {
      const double v = d[r];
      finite = finite && isfinite(v);
      below_abs = below_abs && fabs(v) < fabs(hd->abs[r]);
      below_reach = below_reach && fabs(v) < fabs(reach[(size_t)k * GMG_MAX_S + r]);
    }
    if (!finite) {
      atomicMin(&hd->bad_k, k);
      all = 0;
      continue;
    }
    for (int r = 0; r < s; ++r) last[(size_t)k * GMG_MAX_S + r] = d[r];
    if (below_abs || below_reach) {
      conv[k] = 1;
      iters[k] = it;
    } else {
      all = 0;
    }
  }
  all = __syncthreads_and(all);
  if (threadIdx.x == 0) {
    hd->it = it;
    const bool bad = hd->bad_k < ni;
    if (bad) hd->bad_it = it;
    cudaGraphSetConditional(h, (!bad && !all && it < hd->maxit) ? 1u : 0u);
  }
}

int k_batch_loop_test(gmg_mg *mg, BatchLoopHead *hd, int *iters, double *last, const double *reach,
                      cudaGraphConditionalHandle h) {
  batch_loop_test_kernel<<<1, 1024, 0, mg->stream>>>(hd, mg->batch.norms_dev, mg->batch.conv_dev, iters, last, reach,
                                                     h);
  LAUNCH_CHECK(mg);
  return 0;
}

// daxpy, ugblas.cc:2875: x += a y (per component a), one rounding each
template <class T, int S>
__global__ void __launch_bounds__(BLK) axpy_kernel(long long n, T *__restrict__ x, const T *__restrict__ y,
                                                   Damp<T> a) {
  pdl_prologue();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
#pragma unroll
    for (int r = 0; r < S; ++r) x[i * S + r] = x[i * S + r] + a.d[r] * y[i * S + r];
}

int k_axpy(gmg_mg *mg, int prec, void *x, const void *y, int n, int s, const double *a) {
  if (n <= 0) return 0;
#define AX(TT, SS) GMG_LAUNCH((axpy_kernel<TT, SS>), grid_for(n), BLK, (long long)n, (TT *)x, (const TT *)y, \
                              make_damp<TT>(a, SS))
  if (prec == GMG_PREC_FP64) { if (s == 1) AX(double, 1); else if (s == 2) AX(double, 2); else if (s == 3) AX(double, 3);
                               else { set_error("block size %d not compiled", s); return 1; } }
  else { if (s == 1) AX(float, 1); else if (s == 2) AX(float, 2); else if (s == 3) AX(float, 3);
         else { set_error("block size %d not compiled", s); return 1; } }
#undef AX
  LAUNCH_CHECK(mg);
  return 0;
}

// ------------------------------------------------------------ solution transfer (transgrid.cc:354, 655)
template <class T, int S>
__global__ void __launch_bounds__(BLK) interp_new_kernel(int nf, const int *__restrict__ prow,
                                                         const int *__restrict__ pcol, const double *__restrict__ pw,
                                                         const uint8_t *__restrict__ flags, T *xf,
                                                         const T *__restrict__ xc) {
  pdl_prologue();
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
    if (!(flags[f] & F_VNEW)) continue;
    double acc[S];
#pragma unroll
    for (int r = 0; r < S; ++r) acc[r] = 0.0;
    for (int k = prow[f]; k < prow[f + 1]; ++k) {
      const int c = pcol[k];
      const double w = pw[k];
#pragma unroll
      for (int r = 0; r < S; ++r) acc[r] = __dadd_rn(acc[r], __dmul_rn(w, double(xc[(size_t)c * S + r])));
    }
#pragma unroll
    for (int r = 0; r < S; ++r) xf[(size_t)f * S + r] = T(acc[r]);
  }
}

template <class T, int S>
__global__ void __launch_bounds__(BLK) project_kernel(int nc, const int *__restrict__ son, T *xc,
                                                      const T *__restrict__ xf) {
  pdl_prologue();
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const int f = son[c];
    if (f < 0) continue;
#pragma unroll
    for (int r = 0; r < S; ++r) xc[(size_t)c * S + r] = xf[(size_t)f * S + r];
  }
}

int k_interpolate_new(gmg_mg *mg, const Level &F, int prec, void *xf, const void *xc) {
  if (F.n == 0) return 0;
#define IN(TT, SS) GMG_LAUNCH((interp_new_kernel<TT, SS>), vec_grid(F.n), BLK, F.n, F.P.rowptr, F.P.col, F.P.v64, \
                              F.flags, (TT *)xf, (const TT *)xc)
  if (prec == GMG_PREC_FP64) { if (F.s == 1) IN(double, 1); else if (F.s == 2) IN(double, 2); else if (F.s == 3) IN(double, 3);
                               else { set_error("block size %d not compiled", F.s); return 1; } }
  else { if (F.s == 1) IN(float, 1); else if (F.s == 2) IN(float, 2); else if (F.s == 3) IN(float, 3);
         else { set_error("block size %d not compiled", F.s); return 1; } }
#undef IN
  LAUNCH_CHECK(mg);
  return 0;
}

// InterpolateNewVectorsByMatrix (transgrid.cc:1425-1490): VNEW fine vectors
// take their interpolation-matrix row times the coarse vector, in double with
// unfused products and sums in the row's entry order.  One component: rows
// with a VECSKIP bit keep their value, each entry adds to x directly.
// Blocks: VECSKIP not consulted, per entry the transposed block product
// summed first, then added.
template <class T, int S>
__global__ void __launch_bounds__(BLK) interp_new_imat_kernel(int nf, const int *__restrict__ prow,
                                                              const int *__restrict__ pcol,
                                                              const double *__restrict__ pval,
                                                              const uint8_t *__restrict__ flags,
                                                              const uint8_t *__restrict__ skip, T *xf,
                                                              const T *__restrict__ xc) {
  pdl_prologue();
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
    if (!(flags[f] & F_VNEW)) continue;
    if (S == 1 && skip[f]) continue;
    double v[S];
#pragma unroll
    for (int i = 0; i < S; ++i) v[i] = 0.0;
    for (int k = prow[f]; k < prow[f + 1]; ++k) {
      const double *m = pval + (size_t)k * S * S;
      const T *w = xc + (size_t)pcol[k] * S;
      if (S == 1) {
        v[0] = __dadd_rn(v[0], __dmul_rn(m[0], double(w[0])));
        continue;
      }
#pragma unroll
      for (int i = 0; i < S; ++i) {
        double sum = 0.0;
#pragma unroll
        for (int j = 0; j < S; ++j) sum = __dadd_rn(sum, __dmul_rn(m[j * S + i], double(w[j])));
        v[i] = __dadd_rn(v[i], sum);
      }
    }
#pragma unroll
    for (int i = 0; i < S; ++i) xf[(size_t)f * S + i] = T(v[i]);
  }
}

int k_interpolate_new_imat(gmg_mg *mg, const Level &F, int prec, void *xf, const void *xc) {
  GMG_CHECK(F.has_imat, "InterpolateNewVectorsByMatrix: no interpolation matrix on this level");
  if (F.n == 0) return 0;
#define NI(TT, SS) GMG_LAUNCH((interp_new_imat_kernel<TT, SS>), vec_grid(F.n), BLK, F.n, F.IP.rowptr, F.IP.col, \
                              F.IP.v64, F.flags, F.skip, (TT *)xf, (const TT *)xc)
  if (prec == GMG_PREC_FP64) { if (F.s == 1) NI(double, 1); else if (F.s == 2) NI(double, 2); else if (F.s == 3) NI(double, 3);
                               else { set_error("block size %d not compiled", F.s); return 1; } }
  else { if (F.s == 1) NI(float, 1); else if (F.s == 2) NI(float, 2); else if (F.s == 3) NI(float, 3);
         else { set_error("block size %d not compiled", F.s); return 1; } }
#undef NI
  LAUNCH_CHECK(mg);
  return 0;
}

int k_project(gmg_mg *mg, const Level &F, const Level &C, int prec, void *xc, const void *xf) {
  if (C.n == 0) return 0;
#define PJ(TT, SS) GMG_LAUNCH((project_kernel<TT, SS>), vec_grid(C.n), BLK, C.n, F.son, (TT *)xc, (const TT *)xf)
  if (prec == GMG_PREC_FP64) { if (F.s == 1) PJ(double, 1); else if (F.s == 2) PJ(double, 2); else if (F.s == 3) PJ(double, 3);
                               else { set_error("block size %d not compiled", F.s); return 1; } }
  else { if (F.s == 1) PJ(float, 1); else if (F.s == 2) PJ(float, 2); else if (F.s == 3) PJ(float, 3);
         else { set_error("block size %d not compiled", F.s); return 1; } }
#undef PJ
  LAUNCH_CHECK(mg);
  return 0;
}

// ------------------------------------------------------------ surface of a locally refined hierarchy
// UG's ON_SURFACE loops (np/algebra/vecloop.ct, matloop.ct) visit the
// FINE_GRID_DOF vectors of the levels FULLREFINELEVEL..top-1 and the
// NEW_DEFECT vectors of the top level, each row with its own level's matrix
// and vectors.  One launch covers every level of a SurfLevels table: thread g
// handles row g - row0[l] of the level l with row0[l] <= g < row0[l+1].
// OP 0: b -= A y, 1: b += A y, 2: b = -(A y), 3: b = A y on the selected rows (the
// surface rows of `mask`, or every row where `all` is set)
template <int S, class YT, int OP, bool STREAM>
__global__ void __launch_bounds__(BLK) surf_update_kernel(SurfLevels t) {
  pdl_prologue();
  const int total = t.row0[t.nlev];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    int l = 0;
    while (g >= t.row0[l + 1]) ++l;
    const int i = g - t.row0[l];
    const YT *__restrict__ y = static_cast<const YT *>(t.y[l]);
    if (t.all[l] || (t.mask[l] && (__ldg(t.flags[l] + i) & t.mask[l]))) {
      double acc[S];
#pragma unroll
      for (int r = 0; r < S; ++r) acc[r] = 0.0;
      const int k1 = __ldg(t.rowptr[l] + i + 1);
      for (int k = __ldg(t.rowptr[l] + i); k < k1; ++k) {
        const int j = STREAM ? __ldcs(t.col[l] + k) : __ldg(t.col[l] + k);
        const double *m = t.val[l] + (size_t)k * (S * S);
        double yj[S];
#pragma unroll
        for (int c = 0; c < S; ++c) yj[c] = double(y[(size_t)j * S + c]);
#pragma unroll
        for (int r = 0; r < S; ++r)
#pragma unroll
          for (int c = 0; c < S; ++c) acc[r] = fma(STREAM ? __ldcs(m + r * S + c) : __ldg(m + r * S + c), yj[c], acc[r]);
      }
#pragma unroll
      for (int r = 0; r < S; ++r) {
        double &bv = t.b[l][(size_t)i * S + r];
        bv = OP == 0 ? bv - acc[r] : (OP == 1 ? bv + acc[r] : (OP == 2 ? -acc[r] : acc[r]));
      }
    }
    if (t.addx[l]) {
#pragma unroll
      for (int r = 0; r < S; ++r) t.x[l][(size_t)i * S + r] += double(y[(size_t)i * S + r]);
    }
  }
}

// b32 = b64 on every row of the table's levels; c32 = 0 where zc is set
template <int S>
__global__ void __launch_bounds__(BLK) surf_prepare_kernel(SurfLevels t) {
  pdl_prologue();
  const int total = t.row0[t.nlev];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    int l = 0;
    while (g >= t.row0[l + 1]) ++l;
    const size_t i = size_t(g - t.row0[l]) * S;
#pragma unroll
    for (int r = 0; r < S; ++r) {
      t.b32[l][i + r] = float(t.b[l][i + r]);
      if (t.c32[l]) t.c32[l][i + r] = 0.0f;
    }
  }
}

// dnrm2x ON_SURFACE: per-component sums of squares over the surface rows of
// every level, with the deterministic two-stage reduction of nrm_kernel
template <int S>
__global__ void __launch_bounds__(BLK) surf_nrm_kernel(SurfLevels t, double *__restrict__ partial,
                                                       unsigned *__restrict__ ticket, double *__restrict__ out) {
  pdl_prologue();
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  const int total = t.row0[t.nlev];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    int l = 0;
    while (g >= t.row0[l + 1]) ++l;
    const int i = g - t.row0[l];
    if (!(t.mask[l] && (__ldg(t.flags[l] + i) & t.mask[l]))) continue;
#pragma unroll
    for (int r = 0; r < S; ++r) {
      const double v = t.b[l][(size_t)i * S + r];
      acc[r] = fma(v, v, acc[r]);
    }
  }
  __shared__ double sh[BLK / 32][S];
  __shared__ bool last;
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < S) {
    double v = 0.0;
    for (int w = 0; w < BLK / 32; ++w) v += sh[w][threadIdx.x];
    partial[(size_t)blockIdx.x * S + threadIdx.x] = v;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ double red[BLK];
  for (int r = 0; r < S; ++r) {
    double v = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) v += __ldcg(partial + (size_t)b * S + r);
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[r] = sqrt(red[0]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

int k_surf_update(gmg_mg *mg, const SurfLevels &t, int yprec, int s, int op) {
  if (t.row0[t.nlev] == 0) return 0;
  const int g = vec_grid(t.row0[t.nlev]);
  // an FP32 y is the mixed iteration's correction: the FP64 matrices are then
  // read once per ls iteration while the FP32 cycle reuses its copies, so they
  // stream with evict-first loads
#define SO(SS, OP) { if (yprec == GMG_PREC_FP64) GMG_LAUNCH((surf_update_kernel<SS, double, OP, false>), g, BLK, t); \
                     else GMG_LAUNCH((surf_update_kernel<SS, float, OP, true>), g, BLK, t); }
#define SU(SS) { if (op == 0) SO(SS, 0) else if (op == 1) SO(SS, 1) else if (op == 2) SO(SS, 2) else SO(SS, 3) }
  if (s == 1) SU(1) else if (s == 2) SU(2) else if (s == 3) SU(3)
  else { set_error("block size %d not compiled", s); return 1; }
#undef SU
#undef SO
  LAUNCH_CHECK(mg);
  return 0;
}

// a Krylov dot product over the surface rows of every level (x in t.b, y in
// t.y, FP64), per-component partial sums, the deterministic reduction of
// nrm_kernel, then the solver's scalar step on sc[] (KIND 0: cg's MODE 1 / 2,
// KIND 1: bcgs's BM_* modes)
template <int S, int KIND, int MODE>
__global__ void __launch_bounds__(BLK) surf_dot_kernel(SurfLevels t, double *__restrict__ partial,
                                                       unsigned *__restrict__ ticket, double *__restrict__ sc,
                                                       double sign) {
  pdl_prologue();
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  const int total = t.row0[t.nlev];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    int l = 0;
    while (g >= t.row0[l + 1]) ++l;
    const int i = g - t.row0[l];
    if (!(t.all[l] || (t.mask[l] && (__ldg(t.flags[l] + i) & t.mask[l])))) continue;
    const double *__restrict__ y = static_cast<const double *>(t.y[l]);
#pragma unroll
    for (int r = 0; r < S; ++r) acc[r] = fma(t.b[l][(size_t)i * S + r], y[(size_t)i * S + r], acc[r]);
  }
  __shared__ double sh[BLK / 32][S];
  __shared__ bool last;
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][r] = v;
  }
  __syncthreads();
  if (threadIdx.x < S) {
    double v = 0.0;
    for (int w = 0; w < BLK / 32; ++w) v += sh[w][threadIdx.x];
    partial[(size_t)blockIdx.x * S + threadIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ double red[S][BLK];
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) v += __ldcg(partial + (size_t)b * S + r);
    red[r][threadIdx.x] = v;
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int r = 0; r < S; ++r) red[r][threadIdx.x] += red[r][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double d = 0.0;
    for (int r = 0; r < S; ++r) d += red[r][0];
    if (KIND == 0) cg_scalars<MODE>(sign * d, sc);
    else if (KIND == 1) bcgs_scalars<MODE>(d, sign, sc);
    else sc[0] = sign * d;
    *ticket = 0u;
  }
}

int k_surf_dot(gmg_mg *mg, const SurfLevels &t, int s, int kind, int mode, double sign, double *sc) {
  unsigned *ticket = reinterpret_cast<unsigned *>(mg->norms_dev + GMG_MAX_S);
#define SD(SS, K, M) GMG_LAUNCH((surf_dot_kernel<SS, K, M>), REDUCE_BLOCKS, BLK, t, mg->partial, ticket, sc, sign)
#define SM(SS)                                                                   \
  if (kind == 2) SD(SS, 2, 0);                                                    \
  else if (kind == 0) { if (mode == 1) SD(SS, 0, 1); else SD(SS, 0, 2); }        \
  else if (mode == BM_RHO) SD(SS, 1, BM_RHO); else if (mode == BM_ALPHA) SD(SS, 1, BM_ALPHA); \
  else if (mode == BM_TT) SD(SS, 1, BM_TT); else SD(SS, 1, BM_OMEGA);
  if (s == 1) { SM(1) } else if (s == 2) { SM(2) } else if (s == 3) { SM(3) }
  else { set_error("block size %d not compiled", s); return 1; }
#undef SM
#undef SD
  LAUNCH_CHECK(mg);
  return 0;
}

int k_surf_prepare(gmg_mg *mg, const SurfLevels &t, int s) {
  if (t.row0[t.nlev] == 0) return 0;
  const int g = vec_grid(t.row0[t.nlev]);
  if (s == 1) GMG_LAUNCH((surf_prepare_kernel<1>), g, BLK, t);
  else if (s == 2) GMG_LAUNCH((surf_prepare_kernel<2>), g, BLK, t);
  else if (s == 3) GMG_LAUNCH((surf_prepare_kernel<3>), g, BLK, t);
  else { set_error("block size %d not compiled", s); return 1; }
  LAUNCH_CHECK(mg);
  return 0;
}

int k_surf_nrm2x(gmg_mg *mg, const SurfLevels &t, int s) {
  unsigned *ticket = reinterpret_cast<unsigned *>(mg->norms_dev + GMG_MAX_S);
  if (s == 1) GMG_LAUNCH((surf_nrm_kernel<1>), REDUCE_BLOCKS, BLK, t, mg->partial, ticket, mg->norms_dev);
  else if (s == 2) GMG_LAUNCH((surf_nrm_kernel<2>), REDUCE_BLOCKS, BLK, t, mg->partial, ticket, mg->norms_dev);
  else if (s == 3) GMG_LAUNCH((surf_nrm_kernel<3>), REDUCE_BLOCKS, BLK, t, mg->partial, ticket, mg->norms_dev);
  else { set_error("block size %d not compiled", s); return 1; }
  LAUNCH_CHECK(mg);
  return 0;
}

}  // namespace gmg
