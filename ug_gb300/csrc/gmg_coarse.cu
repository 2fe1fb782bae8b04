// Fused coarse-grid cycle: the lmgc recursion (gamma = 1) over the small
// levels bl..lc, run by ONE thread block out of shared memory.
//
// On the coarse levels a V-cycle is pure latency: each level visit needs
// ~25 dependent phases (smoothing waves, defect updates, dadd, restriction,
// interpolation) of a few hundred rows each, so separate kernel launches or
// grid-wide barriers cost far more than the arithmetic.  Here the matrices,
// transfer operators, schedules and vectors of all levels bl..lc (a few
// hundred KB at most) are copied into shared memory once per cycle, every
// phase of Lmgc (np/procs/iter.cc:7741) is a block-strided loop over a
// level's rows, and phases are separated by __syncthreads.  The arithmetic
// of each phase is that of the per-level kernels in gmg_kernels.cu.
//
// The static data of the fused levels is packed once into a contiguous
// device image (16-byte aligned sections) that the kernel copies with
// 128-bit loads; the vectors b and c of every fused level are read at the
// start and written back at the end (c of the top fused level is the
// coarse-grid correction the caller interpolates; b is written back because
// restriction keeps the old defect on rows with VNCLASS < 2).
//
// On a batched hierarchy every instance is a block of its own on each level,
// so the coarse levels of all instances run at once: one thread block per
// instance, each with an image of its instance's rows only (and a map from
// its rows to the union level's rows for the vectors).  An instance whose
// finest level lies below the fused range runs its whole cycle there,
// starting from its own top level (whose correction it first zeroes, as the
// union cycle's restriction into that level does).
#include <algorithm>
#include <cstring>

#include "gmg_internal.h"
#include "gmg_np.h"

namespace gmg {

namespace {

constexpr int MAXCL = 12;
constexpr int CBLK = 1024;  // threads of the single-hierarchy cycle
constexpr int BBLK = 256;   // threads per instance of the batched cycle
constexpr int NARROW = 128; // threads of the team that runs the smallest levels

// level description: byte offsets into the shared-memory image
struct SLev {
  int n, all_active, nwave, nuwave;
  int o_rowptr, o_col, o_val, o_dinv, o_flags, o_skip;
  int o_lend;  // per row: end of its lower entries (rows stored diagonal | lower | upper)
  int o_wptr, o_wrows, o_uptr, o_urows;
  int o_lrow, o_lcol, o_lval, o_urow, o_ucol, o_uval, o_udinv;
  int o_prow, o_pcol, o_pw, o_rrow, o_rcol, o_rw;
  int o_b, o_c, o_t;  // vectors (after the static image)
  int o_gmap;         // batched: union row of each local row (-1: rows are the level's)
  void *gb, *gc;      // the level's b and c in global memory
};

struct SArgs {
  int nl, nu1, nu2, unit_damp, smem_bytes, image_bytes;
  int zero_top_c;     // batched: zero c on the top fused level first
  int narrow;         // levels 0..narrow-1 run by the first NARROW threads (0: none)
  const int4 *image;  // static part, image_bytes (multiple of 16)
  double damp[GMG_MAX_S], cdamp[GMG_MAX_S], abslimit[GMG_MAX_S];
  int o_ainv, base_dim;
  SLev L[MAXCL];
};

// pointers into shared memory for one level
template <class T>
struct PL {
  int n, all_active, nwave, nuwave;
  const int *rowptr, *lend, *col, *wptr, *wrows, *uptr, *urows, *lrow, *lcol, *urow, *ucol, *prow, *pcol, *rrow,
      *rcol;
  const T *val, *dinv, *lval, *uval, *udinv, *pw, *rw;
  const uint8_t *flags, *skip;
  T *b, *c, *t;
};

template <class T>
__device__ PL<T> make_pl(const SLev &s, char *sm) {
  PL<T> p;
  p.n = s.n; p.all_active = s.all_active; p.nwave = s.nwave; p.nuwave = s.nuwave;
  auto I = [&](int o) { return o >= 0 ? (const int *)(sm + o) : nullptr; };
  auto V = [&](int o) { return o >= 0 ? (const T *)(sm + o) : nullptr; };
  p.rowptr = I(s.o_rowptr); p.lend = I(s.o_lend); p.col = I(s.o_col); p.wptr = I(s.o_wptr);
  p.wrows = I(s.o_wrows);
  p.uptr = I(s.o_uptr); p.urows = I(s.o_urows); p.lrow = I(s.o_lrow); p.lcol = I(s.o_lcol);
  p.urow = I(s.o_urow); p.ucol = I(s.o_ucol); p.prow = I(s.o_prow); p.pcol = I(s.o_pcol);
  p.rrow = I(s.o_rrow); p.rcol = I(s.o_rcol);
  p.val = V(s.o_val); p.dinv = V(s.o_dinv); p.lval = V(s.o_lval); p.uval = V(s.o_uval);
  p.udinv = V(s.o_udinv); p.pw = V(s.o_pw); p.rw = V(s.o_rw);
  p.flags = (const uint8_t *)(sm + s.o_flags); p.skip = (const uint8_t *)(sm + s.o_skip);
  p.b = (T *)(sm + s.o_b); p.c = (T *)(sm + s.o_c); p.t = (T *)(sm + s.o_t);
  return p;
}

template <int S>
struct GL {
  // lanes per row; measured on the C2 cube (one mixed solve): 1 / 2 / 4 / 8
  // lanes 5.36 / 5.36 / 5.44 / 5.52 ms on UG's mesh, 3.09 / 3.13 / 3.19 /
  // 3.30 ms on the Freudenthal triangulation
  static constexpr int G = S == 1 ? 1 : 2;
};

template <int G, class T>
__device__ __forceinline__ T gsum(T v) {
#pragma unroll
  for (int off = G / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// s += sum over the lane's share of `row` of m_k * v_j: the whole row, or
// (LOWER, with the row's lower end `lend`) its strictly lower entries, which
// the image stores right after the diagonal
template <class T, int S, int G, bool LOWER>
__device__ __forceinline__ void row_dot(const int *rowptr, const int *lend, const int *col, const T *val,
                                        const T *v, int row, int first, int lane, bool on, T *s) {
  const int k1 = on ? (LOWER ? lend[row] : rowptr[row + 1]) : 0;
#pragma unroll 4
  for (int k = on ? rowptr[row] + first + lane : 0; k < k1; k += G) {
    const int j = col[k];
    const T *m = val + (size_t)k * S * S;
#pragma unroll
    for (int r = 0; r < S; ++r)
#pragma unroll
      for (int c = 0; c < S; ++c) s[r] = fma(m[r * S + c], v[j * S + c], s[r]);
  }
#pragma unroll
  for (int r = 0; r < S; ++r) s[r] = gsum<G>(s[r]);
}

// the threads running a phase: lanes / groups for the row loops, the team's
// thread index and size for the element loops, and its barrier (0: the whole
// block, __syncthreads; 1: the first nt threads only, a named barrier)
struct Team {
  int lane, grp, ngrp, tid, nt, bar;
};

__device__ __forceinline__ void tsync(const Team &tm) {
  if (tm.bar == 0) __syncthreads();
  else asm volatile("bar.sync %0, %1;\n" ::"r"(tm.bar), "r"(tm.nt) : "memory");
}

// x -= A y ; acc += y (dmatmul_minus + dadd)
template <class T, int S>
__device__ void c_spmv(const PL<T> &L, T *x, const T *y, T *acc, const Team &tm) {
  constexpr int G = GL<S>::G;
  for (int base = 0; base < L.n; base += tm.ngrp) {
    const int i = base + tm.grp;
    const bool valid = i < L.n;
    const bool own = valid && tm.lane == 0;
    // the row's own entries first: they do not wait for the gathers
    T xi[S], yi[S], ai[S];
#pragma unroll
    for (int r = 0; r < S; ++r) {
      xi[r] = own ? x[i * S + r] : T(0);
      yi[r] = own && acc ? y[i * S + r] : T(0);
      ai[r] = own && acc ? acc[i * S + r] : T(0);
    }
    T s[S];
#pragma unroll
    for (int r = 0; r < S; ++r) s[r] = T(0);
    row_dot<T, S, G, false>(L.rowptr, L.lend, L.col, L.val, y, i, 0, tm.lane, valid, s);
    if (own) {
#pragma unroll
      for (int r = 0; r < S; ++r) {
        x[i * S + r] = xi[r] - s[r];
        if (acc) acc[i * S + r] = ai[r] + yi[r];
      }
    }
  }
}

// t = damp * D^{-1} b (l_jac + dscalx)
template <class T, int S>
__device__ void c_jac(const PL<T> &L, const SArgs &a, const Team &tm) {
  for (int i = tm.tid; i < L.n; i += tm.nt) {
    if (!L.all_active && !(L.flags[i] & F_ACTIVE)) {
#pragma unroll
      for (int r = 0; r < S; ++r) L.t[i * S + r] = T(0);
      continue;
    }
#pragma unroll
    for (int r = 0; r < S; ++r) {
      T v = T(0);
#pragma unroll
      for (int c = 0; c < S; ++c) v = fma(L.dinv[i * S * S + r * S + c], L.b[i * S + c], v);
      L.t[i * S + r] = v * T(a.damp[r]);
    }
  }
}

// (D+L) t = b over the wavefronts (l_lgs)
template <class T, int S>
__device__ void c_gs(const PL<T> &L, const Team &tm) {
  constexpr int G = GL<S>::G;
  for (int w = 0; w < L.nwave; ++w) {
    const int r0 = L.wptr[w], r1 = L.wptr[w + 1];
    for (int base = r0; base < r1; base += tm.ngrp) {
      const int q = base + tm.grp;
      const bool valid = q < r1;
      const int i = valid ? L.wrows[q] : 0;
      const bool act = valid && (L.all_active || (L.flags[i] & F_ACTIVE));
      const bool own = valid && tm.lane == 0;
      // b and the inverse diagonal of the row before the gathers
      T bi[S], di[S * S];
#pragma unroll
      for (int r = 0; r < S; ++r) bi[r] = own ? L.b[i * S + r] : T(0);
#pragma unroll
      for (int k = 0; k < S * S; ++k) di[k] = own ? L.dinv[i * S * S + k] : T(0);
      T s[S];
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = T(0);
      row_dot<T, S, G, true>(L.rowptr, L.lend, L.col, L.val, L.t, i, 1, tm.lane, act, s);
      if (own) {
        T rhs[S];
#pragma unroll
        for (int r = 0; r < S; ++r) rhs[r] = bi[r] - s[r];
#pragma unroll
        for (int r = 0; r < S; ++r) {
          T v = T(0);
#pragma unroll
          for (int c = 0; c < S; ++c) v = fma(di[r * S + c], rhs[c], v);
          L.t[i * S + r] = act ? v : T(0);
        }
      }
    }
    tsync(tm);
  }
}

// L U t = b (l_luiter)
template <class T, int S>
__device__ void c_ilu(const PL<T> &L, const Team &tm) {
  constexpr int G = GL<S>::G;
  for (int w = 0; w < L.nwave; ++w) {
    const int r0 = L.wptr[w], r1 = L.wptr[w + 1];
    for (int base = r0; base < r1; base += tm.ngrp) {
      const int q = base + tm.grp;
      const bool valid = q < r1;
      const int i = valid ? L.wrows[q] : 0;
      const bool act = valid && (L.all_active || (L.flags[i] & F_ACTIVE));
      T s[S];
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = T(0);
      row_dot<T, S, G, false>(L.lrow, nullptr, L.lcol, L.lval, L.t, i, 0, tm.lane, act, s);
      if (valid && tm.lane == 0)
#pragma unroll
        for (int r = 0; r < S; ++r) L.t[i * S + r] = act ? L.b[i * S + r] - s[r] : T(0);
    }
    tsync(tm);
  }
  for (int w = 0; w < L.nuwave; ++w) {
    const int r0 = L.uptr[w], r1 = L.uptr[w + 1];
    for (int base = r0; base < r1; base += tm.ngrp) {
      const int q = base + tm.grp;
      const bool valid = q < r1;
      const int i = valid ? L.urows[q] : 0;
      const bool act = valid && (L.all_active || (L.flags[i] & F_ACTIVE));
      T s[S];
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = T(0);
      row_dot<T, S, G, false>(L.urow, nullptr, L.ucol, L.uval, L.t, i, 0, tm.lane, act, s);
      if (act && tm.lane == 0) {
        T rhs[S];
#pragma unroll
        for (int r = 0; r < S; ++r) rhs[r] = L.t[i * S + r] - s[r];
#pragma unroll
        for (int r = 0; r < S; ++r) {
          T v = T(0);
#pragma unroll
          for (int c = 0; c < S; ++c) v = fma(L.udinv[i * S * S + r * S + c], rhs[c], v);
          L.t[i * S + r] = v;
        }
      }
    }
    tsync(tm);
  }
}

// one step of Smoother (iter.cc:817) followed by lmgc's dadd(c, t)
template <class T, int S, int SMO>
__device__ void c_smooth(const PL<T> &L, const SArgs &a, const Team &tm) {
  if (SMO == 0) {
    c_jac<T, S>(L, a, tm);
    tsync(tm);
  } else {
    if (SMO == 1) c_gs<T, S>(L, tm);
    else c_ilu<T, S>(L, tm);
    if (!a.unit_damp) {
      for (int i = tm.tid; i < L.n; i += tm.nt)
#pragma unroll
        for (int r = 0; r < S; ++r) L.t[i * S + r] *= T(a.damp[r]);
      tsync(tm);
    }
  }
  c_spmv<T, S>(L, L.b, L.t, L.c, tm);
  tsync(tm);
}

// StandardRestrict into the level below, fused with lmgc's dset(c_{l-1}, 0)
template <class T, int S>
__device__ void c_restrict(const PL<T> &F, const PL<T> &Cl, const Team &tm) {
  for (int c = tm.tid; c < Cl.n; c += tm.nt) {
    const bool reset = Cl.flags[c] & F_RESET;
    const int sk = Cl.skip[c];
    T acc[S];
#pragma unroll
    for (int r = 0; r < S; ++r) acc[r] = reset ? T(0) : Cl.b[c * S + r];
    for (int k = F.rrow[c]; k < F.rrow[c + 1]; ++k) {
      const int f = F.rcol[k];
      const T w = F.rw[k];
#pragma unroll
      for (int r = 0; r < S; ++r) acc[r] = fma(w, F.b[f * S + r], acc[r]);
    }
#pragma unroll
    for (int r = 0; r < S; ++r) {
      if (!(sk & (1 << r))) Cl.b[c * S + r] = acc[r];
      else if (reset) Cl.b[c * S + r] = T(0);
      Cl.c[c * S + r] = T(0);
    }
  }
}

// StandardInterpolateCorrection into t, fused with lmgc's dadd(c, t)
template <class T, int S>
__device__ void c_interp(const PL<T> &F, const PL<T> &Cl, const SArgs &a, const Team &tm) {
  for (int f = tm.tid; f < F.n; f += tm.nt) {
    const int sk = F.skip[f];
    T v[S];
#pragma unroll
    for (int r = 0; r < S; ++r) v[r] = T(0);
    if (sk != (1 << S) - 1) {
      for (int k = F.prow[f]; k < F.prow[f + 1]; ++k) {
        const int c = F.pcol[k];
        const T w = F.pw[k];
#pragma unroll
        for (int r = 0; r < S; ++r) v[r] = fma(w * T(a.cdamp[r]), Cl.c[c * S + r], v[r]);
      }
#pragma unroll
      for (int r = 0; r < S; ++r)
        if (sk & (1 << r)) v[r] = T(0);
    }
#pragma unroll
    for (int r = 0; r < S; ++r) {
      F.t[f * S + r] = v[r];
      F.c[f * S + r] += v[r];
    }
  }
}

// base solver `ls $m 1 $I ex`: skip below the abslimit, else t = A^{-1} b; b -= A t; c += t
template <class T, int S>
__device__ void c_base(const PL<T> &B, const SArgs &a, const double *ainv, const Team &tm) {
  __shared__ double red[S][CBLK / 32];
  __shared__ int skip;
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (int i = tm.tid; i < B.n; i += tm.nt)
#pragma unroll
    for (int r = 0; r < S; ++r) {
      double v = double(B.b[i * S + r]);
      acc[r] += v * v;
    }
#pragma unroll
  for (int r = 0; r < S; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((tm.tid & 31) == 0) red[r][tm.tid >> 5] = v;
  }
  tsync(tm);
  if (tm.tid == 0) {
    int below = 1;
    for (int r = 0; r < S; ++r) {
      double v = 0.0;
      for (int w = 0; w < (int)(tm.nt / 32); ++w) v += red[r][w];
      if (fabs(sqrt(v)) >= fabs(a.abslimit[r])) below = 0;
    }
    skip = below;
  }
  tsync(tm);
  if (skip) return;
  const int N = B.n * S;
  for (int i = tm.tid; i < N; i += tm.nt) {
    double v = 0.0;
    for (int j = 0; j < N; ++j) v = fma(ainv[i * N + j], double(B.b[j]), v);
    B.t[i] = T(v);
  }
  tsync(tm);
  c_spmv<T, S>(B, B.b, B.t, B.c, tm);
  tsync(tm);
}

// the cycle over the fused levels, shared memory `sm` holding a's image
template <class T, int S, int SMO>
__device__ void cycle_body(const SArgs &a, char *sm) {
  int4 *smem4 = reinterpret_cast<int4 *>(sm);
  // static image: 128-bit copies, eight loads in flight per thread
  {
    const int nv = a.image_bytes / 16, bd = blockDim.x;
    int i = threadIdx.x;
    for (; i + 7 * bd < nv; i += 8 * bd) {
      int4 r[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) r[u] = __ldg(a.image + i + u * bd);
#pragma unroll
      for (int u = 0; u < 8; ++u) smem4[i + u * bd] = r[u];
    }
    for (; i < nv; i += bd) smem4[i] = __ldg(a.image + i);
  }
  __syncthreads();
  // vectors: b and c of every fused level (through the row map when batched)
  for (int k = 0; k < a.nl; ++k) {
    const SLev &s = a.L[k];
    T *b = (T *)(sm + s.o_b), *c = (T *)(sm + s.o_c);
    const T *gb = (const T *)s.gb, *gc = (const T *)s.gc;
    const int *gm = s.o_gmap >= 0 ? (const int *)(sm + s.o_gmap) : nullptr;
    const bool zc = a.zero_top_c && k == a.nl - 1;
    for (int i = threadIdx.x; i < s.n * S; i += blockDim.x) {
      const size_t g = gm ? (size_t)gm[i / S] * S + i % S : (size_t)i;
      b[i] = gb[g];
      c[i] = zc ? T(0) : gc[g];
    }
  }
  __syncthreads();
  constexpr int G = GL<S>::G;
  const Team wide{int(threadIdx.x & (G - 1)), int(threadIdx.x / G), int(blockDim.x / G), int(threadIdx.x),
                  int(blockDim.x), 0};
  // the bottom levels 0..nn-1 (a few rows each) belong to a team of the first
  // NARROW threads with its own barrier: the other warps skip their phases
  // instead of passing ~25 block-wide barriers per level with nothing to do
  const int nn = a.narrow;
  const Team nar{int(threadIdx.x & (G - 1)), int(threadIdx.x / G), NARROW / G, int(threadIdx.x), NARROW, 1};
  auto down = [&](int k, const Team &tm) {  // pre-smoothing and restriction
    const PL<T> L = make_pl<T>(a.L[k], sm);
    for (int it = 0; it < a.nu1; ++it) c_smooth<T, S, SMO>(L, a, tm);
    c_restrict<T, S>(L, make_pl<T>(a.L[k - 1], sm), tm);
    tsync(tm);
  };
  auto up = [&](int k, const Team &tm) {  // interpolation, coarse-grid correction, post-smoothing
    const PL<T> L = make_pl<T>(a.L[k], sm);
    c_interp<T, S>(L, make_pl<T>(a.L[k - 1], sm), a, tm);
    tsync(tm);
    c_spmv<T, S>(L, L.b, L.t, nullptr, tm);
    tsync(tm);
    for (int it = 0; it < a.nu2; ++it) c_smooth<T, S, SMO>(L, a, tm);
  };
  const double *ainv = reinterpret_cast<const double *>(sm + a.o_ainv);
  const int k0 = nn > 1 ? nn : 1;  // lowest level visited by the whole block
  for (int k = a.nl - 1; k >= k0; --k) down(k, wide);
  if (nn > 0) {
    if (threadIdx.x < NARROW) {
      for (int k = nn - 1; k >= 1; --k) down(k, nar);
      c_base<T, S>(make_pl<T>(a.L[0], sm), a, ainv, nar);
      for (int k = 1; k < nn; ++k) up(k, nar);
    }
    __syncthreads();
  } else {
    c_base<T, S>(make_pl<T>(a.L[0], sm), a, ainv, wide);
  }
  for (int k = k0; k < a.nl; ++k) up(k, wide);
  // write back b and c of every fused level
  for (int k = 0; k < a.nl; ++k) {
    const SLev &s = a.L[k];
    const T *b = (const T *)(sm + s.o_b), *c = (const T *)(sm + s.o_c);
    T *gb = (T *)s.gb, *gc = (T *)s.gc;
    const int *gm = s.o_gmap >= 0 ? (const int *)(sm + s.o_gmap) : nullptr;
    for (int i = threadIdx.x; i < s.n * S; i += blockDim.x) {
      const size_t g = gm ? (size_t)gm[i / S] * S + i % S : (size_t)i;
      gb[g] = b[i];
      gc[g] = c[i];
    }
  }
}

template <class T, int S, int SMO>
__global__ void __launch_bounds__(CBLK, 1) coarse_cycle_kernel(const __grid_constant__ SArgs a) {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");  // programmatic dependent launch
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  extern __shared__ int4 smem4[];
  cycle_body<T, S, SMO>(a, reinterpret_cast<char *>(smem4));
}

// per-call parameters of the batched cycle (the same for every instance)
struct BCall {
  int nu1, nu2, unit_damp;
  double damp[GMG_MAX_S], cdamp[GMG_MAX_S], abslimit[GMG_MAX_S];
  void *gb[MAXCL], *gc[MAXCL];  // union vectors of levels bl..lc
  int bl;
};

// one block per instance; args[k] describes instance k's fused levels
template <class T, int S, int SMO>
__global__ void __launch_bounds__(BBLK) coarse_cycle_batched_kernel(const SArgs *__restrict__ args,
                                                                    const __grid_constant__ BCall call) {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  extern __shared__ int4 smem4[];
  __shared__ SArgs a;
  {
    const int *src = reinterpret_cast<const int *>(args + blockIdx.x);
    int *dst = reinterpret_cast<int *>(&a);
    for (int i = threadIdx.x; i < int(sizeof(SArgs) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a.nu1 = call.nu1;
    a.nu2 = call.nu2;
    a.unit_damp = call.unit_damp;
    for (int r = 0; r < GMG_MAX_S; ++r) {
      a.damp[r] = call.damp[r];
      a.cdamp[r] = call.cdamp[r];
      a.abslimit[r] = call.abslimit[r];
    }
    for (int k = 0; k < a.nl; ++k) {
      a.L[k].gb = call.gb[k];
      a.L[k].gc = call.gc[k];
    }
  }
  __syncthreads();
  cycle_body<T, S, SMO>(a, reinterpret_cast<char *>(smem4));
}

// ---------------------------------------------------------------- host: the image
struct Image {
  std::vector<char> host;
  int add(const void *p, size_t bytes) {
    if (!p || bytes == 0) return -1;
    size_t o = (host.size() + 15) & ~size_t(15);
    host.resize(o + ((bytes + 15) & ~size_t(15)), 0);
    std::memcpy(host.data() + o, p, bytes);
    return int(o);
  }
};

template <class T>
std::vector<T> conv(const std::vector<double> &d) {
  return std::vector<T>(d.begin(), d.end());
}

template <class T>
static int d2h(std::vector<T> &out, const T *dev, size_t n) {
  out.resize(n);
  if (n) GMG_CUDA(cudaMemcpy(out.data(), dev, n * sizeof(T), cudaMemcpyDeviceToHost));
  return 0;
}

// host copies of one level's device-only arrays, the input of the images
struct LevelHost {
  std::vector<double> dinv, Lv, Uv, Ud, pw, rw, ainv;
  std::vector<int> lrows, urows, Lrp, Lcol, Urp, Ucol, prp, pcol, rrp, rcol;
  std::vector<long long> aoff;  // block inverses (batched base level)
};

static int fetch_level(gmg_mg *mg, int l, bool ilu, bool transfer, bool base, LevelHost &H) {
  const Level &L = mg->lev[l];
  const int ss = L.s * L.s;
  if (d2h(H.dinv, L.dinv64, size_t(L.n) * ss) || d2h(H.lrows, L.lower.rows, L.n) || d2h(H.urows, L.upper.rows, L.n))
    return 1;
  if (ilu) {
    GMG_CHECK(L.ilu_ready, "ILU factors missing on level %d", l);
    if (d2h(H.Lrp, L.L.rowptr, L.n + 1) || d2h(H.Lcol, L.L.col, L.L.nnz) || d2h(H.Urp, L.U.rowptr, L.n + 1) ||
        d2h(H.Ucol, L.U.col, L.U.nnz) || d2h(H.Lv, L.L.v64, L.L.nnz * ss) || d2h(H.Uv, L.U.v64, L.U.nnz * ss) ||
        d2h(H.Ud, L.udinv64, size_t(L.n) * ss))
      return 1;
  }
  if (transfer) {
    if (d2h(H.prp, L.P.rowptr, L.n + 1) || d2h(H.pcol, L.P.col, L.P.nnz) || d2h(H.pw, L.P.v64, L.P.nnz) ||
        d2h(H.rrp, L.R.rowptr, mg->lev[l - 1].n + 1) || d2h(H.rcol, L.R.col, L.R.nnz) || d2h(H.rw, L.R.v64, L.R.nnz))
      return 1;
  }
  if (base) {
    GMG_CHECK(L.ainv, "base level inverse not computed (ex PreProcess)");
    if (L.nblk_dev > 0) {
      size_t tot = 0;
      for (int b = 0; b < L.nblk_dev; ++b) {
        const size_t N = size_t(L.blk_ptr[b + 1] - L.blk_ptr[b]) * L.s;
        H.aoff.push_back((long long)tot);
        tot += N * N;
      }
      if (d2h(H.ainv, L.ainv, tot)) return 1;
    } else if (d2h(H.ainv, L.ainv, size_t(L.base_dim) * L.base_dim)) {
      return 1;
    }
  }
  return 0;
}

// rows of a CSR-like structure restricted to `rows`, columns renumbered by
// `loc` (-1: not in the subset, entry dropped -- never happens for blocks)
static void sub_csr(const std::vector<int> &rp, const std::vector<int> &col, const std::vector<int> &rows,
                    const std::vector<int> &loc, std::vector<int> &orp, std::vector<int> &ocol,
                    std::vector<int> &src) {
  orp.assign(1, 0);
  ocol.clear();
  src.clear();
  for (int i : rows) {
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      const int j = loc[col[k]];
      if (j < 0) continue;
      ocol.push_back(j);
      src.push_back(k);
    }
    orp.push_back(int(ocol.size()));
  }
}

template <class T>
static std::vector<T> gather_blocks(const double *v, const std::vector<int> &idx, int ss) {
  std::vector<T> o(idx.size() * ss);
  for (size_t q = 0; q < idx.size(); ++q)
    for (int e = 0; e < ss; ++e) o[q * ss + e] = T(v[size_t(idx[q]) * ss + e]);
  return o;
}

// schedule restricted to the subset: the wavefronts that keep rows, local numbers
static void sub_sched(const std::vector<int> &ptr, const std::vector<int> &rows, const std::vector<int> &loc,
                      std::vector<int> &optr, std::vector<int> &orows) {
  optr.assign(1, 0);
  orows.clear();
  for (size_t w = 0; w + 1 < ptr.size(); ++w) {
    for (int q = ptr[w]; q < ptr[w + 1]; ++q)
      if (loc[rows[q]] >= 0) orows.push_back(loc[rows[q]]);
    if (int(orows.size()) > optr.back()) optr.push_back(int(orows.size()));
  }
}

// The image of levels bl..bl+nl-1 restricted to the rows `sub[k]` of each
// (processing order; each a closed block of the level), `gmap` the union
// rows to record (batched) or not (all rows of the levels).  `base_blk` is
// the block of the base level's inverse (-1: the whole-level inverse).
template <class T>
int build_image(gmg_mg *mg, int bl, int nl, int smo, const std::vector<LevelHost> &LH,
                const std::vector<std::vector<int>> &sub, bool gmap, int base_blk, SArgs &a, std::vector<char> &img,
                int *smem_total) {
  Image im;
  const int s = mg->lev[bl].s, ss = s * s;
  a.nl = nl;
  GMG_CHECK(a.nl >= 1 && a.nl <= MAXCL, "fused coarse cycle: %d levels (max %d)", a.nl, MAXCL);
  std::vector<std::vector<int>> loc(nl);
  for (int k = 0; k < nl; ++k) {
    loc[k].assign(mg->lev[bl + k].n, -1);
    for (size_t q = 0; q < sub[k].size(); ++q) loc[k][sub[k][q]] = int(q);
  }
  std::vector<int> rp, cl, src, ptr, rows;
  for (int k = 0; k < nl; ++k) {
    const Level &L = mg->lev[bl + k];
    const LevelHost &H = LH[k];
    const std::vector<int> &R = sub[k];
    const int n = int(R.size());
    SLev &d = a.L[k];
    std::memset(&d, 0xff, sizeof d);  // all offsets -1
    d.n = n;
    bool all = true;
    std::vector<uint8_t> fl(n), sk(n);
    for (int q = 0; q < n; ++q) {
      fl[q] = L.h_flags[R[q]];
      sk[q] = L.h_skip[R[q]];
      all = all && (fl[q] & F_ACTIVE);
    }
    d.all_active = all;
    sub_csr(L.h_rowptr, L.h_col, R, loc[k], rp, cl, src);
    {  // every row as diagonal | strictly lower | upper, each part in stored order
      std::vector<int> c2(cl.size()), s2(src.size()), lend(n);
      for (int q = 0; q < n; ++q) {
        int o = rp[q];
        for (int part = 0; part < 3; ++part) {
          for (int e = rp[q]; e < rp[q + 1]; ++e) {
            const int p = cl[e] == q ? 0 : (cl[e] < q ? 1 : 2);
            if (p != part) continue;
            c2[o] = cl[e];
            s2[o] = src[e];
            ++o;
          }
          if (part == 1) lend[q] = o;
        }
      }
      cl.swap(c2);
      src.swap(s2);
      d.o_lend = im.add(lend.data(), lend.size() * 4);
    }
    d.o_rowptr = im.add(rp.data(), rp.size() * 4);
    d.o_col = im.add(cl.data(), cl.size() * 4);
    auto v = gather_blocks<T>(L.h_val.data(), src, ss);
    d.o_val = im.add(v.data(), v.size() * sizeof(T));
    auto dv = gather_blocks<T>(H.dinv.data(), R, ss);
    d.o_dinv = im.add(dv.data(), dv.size() * sizeof(T));
    d.o_flags = im.add(fl.data(), n);
    d.o_skip = im.add(sk.data(), n);
    sub_sched(L.lower.ptr, H.lrows, loc[k], ptr, rows);
    d.nwave = int(ptr.size()) - 1;
    d.o_wptr = im.add(ptr.data(), ptr.size() * 4);
    d.o_wrows = im.add(rows.data(), rows.size() * 4);
    sub_sched(L.upper.ptr, H.urows, loc[k], ptr, rows);
    d.nuwave = int(ptr.size()) - 1;
    d.o_uptr = im.add(ptr.data(), ptr.size() * 4);
    d.o_urows = im.add(rows.data(), rows.size() * 4);
    if (smo == 2 && k > 0) {
      sub_csr(H.Lrp, H.Lcol, R, loc[k], rp, cl, src);
      d.o_lrow = im.add(rp.data(), rp.size() * 4);
      d.o_lcol = im.add(cl.data(), cl.size() * 4);
      auto lt = gather_blocks<T>(H.Lv.data(), src, ss);
      d.o_lval = im.add(lt.data(), lt.size() * sizeof(T));
      sub_csr(H.Urp, H.Ucol, R, loc[k], rp, cl, src);
      d.o_urow = im.add(rp.data(), rp.size() * 4);
      d.o_ucol = im.add(cl.data(), cl.size() * 4);
      auto ut = gather_blocks<T>(H.Uv.data(), src, ss);
      d.o_uval = im.add(ut.data(), ut.size() * sizeof(T));
      auto udt = gather_blocks<T>(H.Ud.data(), R, ss);
      d.o_udinv = im.add(udt.data(), udt.size() * sizeof(T));
    }
    if (k > 0) {  // transfer from the level below
      sub_csr(H.prp, H.pcol, R, loc[k - 1], rp, cl, src);
      d.o_prow = im.add(rp.data(), rp.size() * 4);
      d.o_pcol = im.add(cl.data(), cl.size() * 4);
      auto pt = gather_blocks<T>(H.pw.data(), src, 1);
      d.o_pw = im.add(pt.data(), pt.size() * sizeof(T));
      sub_csr(H.rrp, H.rcol, sub[k - 1], loc[k], rp, cl, src);
      d.o_rrow = im.add(rp.data(), rp.size() * 4);
      d.o_rcol = im.add(cl.data(), cl.size() * 4);
      auto rt = gather_blocks<T>(H.rw.data(), src, 1);
      d.o_rw = im.add(rt.data(), rt.size() * sizeof(T));
    }
    if (gmap) d.o_gmap = im.add(R.data(), R.size() * 4);
  }
  const LevelHost &HB = LH[0];
  if (base_blk < 0) {
    const Level &B = mg->lev[bl];
    GMG_CHECK(B.base_dim == B.n * s, "base level inverse not computed (ex PreProcess)");
    a.o_ainv = im.add(HB.ainv.data(), HB.ainv.size() * 8);
    a.base_dim = B.base_dim;
  } else {
    const size_t N = sub[0].size() * s;
    a.o_ainv = im.add(HB.ainv.data() + HB.aoff[base_blk], N * N * 8);
    a.base_dim = int(N);
  }
  a.image_bytes = int((im.host.size() + 15) & ~size_t(15));
  im.host.resize(a.image_bytes, 0);
  // vectors after the image
  size_t off = im.host.size();
  for (int k = 0; k < a.nl; ++k) {
    const size_t vb = ((sub[k].size() * s * sizeof(T)) + 15) & ~size_t(15);
    a.L[k].o_b = int(off); off += vb;
    a.L[k].o_c = int(off); off += vb;
    a.L[k].o_t = int(off); off += vb;
  }
  *smem_total = int(off);
  img.swap(im.host);
  return 0;
}

struct CachedImage : CoarseImageBase {
  int bl = -1, lc = -1, prec = -1, smo = -1;
  bool batched = false;
  void *dev = nullptr;        // images (all instances)
  SArgs *dev_args = nullptr;  // batched: per-instance descriptors
  SArgs args{};               // single: the descriptor
  int smem = 0;               // largest per-block shared memory
  int ninst = 0;
  ~CachedImage() override {
    if (dev) cudaFree(dev);
    if (dev_args) cudaFree(dev_args);
  }
};

// single hierarchy: the whole levels
template <class T>
static int make_single(gmg_mg *mg, int bl, int lc, int smo, CachedImage &e) {
  const int nl = lc - bl + 1;
  std::vector<LevelHost> LH(nl);
  std::vector<std::vector<int>> sub(nl);
  for (int k = 0; k < nl; ++k) {
    if (fetch_level(mg, bl + k, smo == 2 && k > 0, k > 0, k == 0, LH[k])) return 1;
    sub[k].resize(mg->lev[bl + k].n);
    for (int i = 0; i < mg->lev[bl + k].n; ++i) sub[k][i] = i;
  }
  std::vector<char> img;
  if (build_image<T>(mg, bl, nl, smo, LH, sub, false, -1, e.args, img, &e.smem)) return 1;
  {  // the narrow team takes the levels from the base up with at most ~4 rows per lane group
    const int G = mg->lev[bl].s == 1 ? GL<1>::G : GL<2>::G;
    int nn = 0;
    while (nn < nl && e.args.L[nn].n <= 4 * (NARROW / G)) ++nn;
    e.args.narrow = nn;
  }
  GMG_CHECK(e.smem <= 227 * 1024, "fused coarse cycle needs %d bytes of shared memory", e.smem);
  GMG_CUDA(cudaMalloc(&e.dev, img.size()));
  GMG_CUDA(cudaMemcpy(e.dev, img.data(), img.size(), cudaMemcpyHostToDevice));
  e.args.image = (const int4 *)e.dev;
  e.args.smem_bytes = e.smem;
  e.args.zero_top_c = 0;
  return 0;
}

// batched hierarchy: instance k's rows on levels bl..min(lc, top_k)
template <class T>
static int make_batched(gmg_mg *mg, int bl, int lc, int smo, bool upload, CachedImage &e) {
  const auto &B = mg->batch;
  const int nl = lc - bl + 1;
  std::vector<LevelHost> LH(nl);
  for (int k = 0; k < nl; ++k)
    if (fetch_level(mg, bl + k, smo == 2 && k > 0, k > 0, k == 0, LH[k])) return 1;
  std::vector<SArgs> args(B.ninst);
  std::vector<char> all;
  std::vector<size_t> img_off(B.ninst);
  e.smem = 0;
  for (int id = 0; id < B.ninst; ++id) {
    const int tf = std::min(lc, B.top[id]);
    GMG_CHECK(tf >= bl, "instance %d: finest level %d below the base level %d", id, B.top[id], bl);
    const int inl = tf - bl + 1;
    std::vector<std::vector<int>> sub(inl);
    for (int k = 0; k < inl; ++k) {
      const Level &L = mg->lev[bl + k];
      // instance id's block on this level: blocks are in instance order over
      // the instances present, and every instance has the levels up to its top
      int blk = 0;
      for (int j = 0; j < id; ++j) blk += B.top[j] >= bl + k;
      sub[k].assign(L.blk_rows.begin() + L.blk_ptr[blk], L.blk_rows.begin() + L.blk_ptr[blk + 1]);
    }
    int base_blk = 0;
    for (int j = 0; j < id; ++j) base_blk += B.top[j] >= bl;
    std::vector<char> img;
    int smem = 0;
    SArgs &a = args[id];
    std::memset(&a, 0, sizeof a);
    if (build_image<T>(mg, bl, inl, smo, LH, sub, true, base_blk, a, img, &smem)) return 1;
    a.smem_bytes = smem;
    a.zero_top_c = tf < lc;
    e.smem = std::max(e.smem, smem);
    img_off[id] = all.size();
    all.insert(all.end(), img.begin(), img.end());
  }
  e.ninst = B.ninst;
  if (!upload) return 0;
  GMG_CHECK(e.smem <= 227 * 1024, "batched fused coarse cycle needs %d bytes of shared memory", e.smem);
  GMG_CUDA(cudaMalloc(&e.dev, all.size()));
  GMG_CUDA(cudaMemcpy(e.dev, all.data(), all.size(), cudaMemcpyHostToDevice));
  for (int id = 0; id < B.ninst; ++id) args[id].image = (const int4 *)((char *)e.dev + img_off[id]);
  GMG_CUDA(cudaMalloc(&e.dev_args, sizeof(SArgs) * B.ninst));
  GMG_CUDA(cudaMemcpy(e.dev_args, args.data(), sizeof(SArgs) * B.ninst, cudaMemcpyHostToDevice));
  return 0;
}

// the cached images of (bl, lc, prec, smo), built on first use (an eager,
// uncaptured call: building copies device data to the host)
static CachedImage *get_image(gmg_mg *mg, int bl, int lc, int prec, int smo, int *err) {
  *err = 0;
  const bool batched = mg->batch.ninst > 0;
  for (auto &b0 : mg->coarse_images) {
    CachedImage *e = static_cast<CachedImage *>(b0.get());
    if (e->bl == bl && e->lc == lc && e->prec == prec && e->smo == smo && e->batched == batched) return e;
  }
  auto e = std::make_unique<CachedImage>();
  e->bl = bl; e->lc = lc; e->prec = prec; e->smo = smo; e->batched = batched;
  int rc;
  if (batched)
    rc = prec == GMG_PREC_FP64 ? make_batched<double>(mg, bl, lc, smo, true, *e)
                               : make_batched<float>(mg, bl, lc, smo, true, *e);
  else
    rc = prec == GMG_PREC_FP64 ? make_single<double>(mg, bl, lc, smo, *e) : make_single<float>(mg, bl, lc, smo, *e);
  if (rc) { *err = 1; return nullptr; }
  CachedImage *r = e.get();
  mg->coarse_images.push_back(std::move(e));
  return r;
}

}  // namespace

// shared-memory bytes the fused cycle needs for levels bl..lc (no device work;
// for a batched hierarchy: the largest instance's, from its exact image)
long long coarse_smem_bytes(const gmg_mg *mg_c, int bl, int lc, int prec, int smo) {
  gmg_mg *mg = const_cast<gmg_mg *>(mg_c);
  if (mg->batch.ninst > 0) {
    const auto key = std::make_tuple(bl, lc, prec, smo);
    auto it = mg->coarse_smem_cache.find(key);
    if (it != mg->coarse_smem_cache.end()) return it->second;
    // a lower bound first (the matrices of the largest instance), so that
    // ranges far above any shared-memory size build no images
    const auto &B = mg->batch;
    const size_t T = prec == GMG_PREC_FP64 ? 8 : 4, ss = size_t(mg->lev[bl].s) * mg->lev[bl].s;
    long long lb = 0;
    for (int l = bl; l <= lc; ++l) {
      const Level &L = mg->lev[l];
      for (int b = 0; b + 1 < (int)L.blk_ptr.size(); ++b) {
        long long nnz = 0;
        for (int q = L.blk_ptr[b]; q < L.blk_ptr[b + 1]; ++q) nnz += L.h_rowptr[L.blk_rows[q] + 1] - L.h_rowptr[L.blk_rows[q]];
        lb = std::max(lb, nnz * (long long)(4 + ss * T));
      }
    }
    (void)B;
    long long r = lb;
    if (lb <= 227 * 1024) {
      CachedImage probe;
      int rc = prec == GMG_PREC_FP64 ? make_batched<double>(mg, bl, lc, smo, false, probe)
                                     : make_batched<float>(mg, bl, lc, smo, false, probe);
      r = rc ? (1LL << 40) : probe.smem;
    }
    mg->coarse_smem_cache[key] = r;
    return r;
  }
  const int s = mg->lev[bl].s, ss = s * s;
  const size_t T = prec == GMG_PREC_FP64 ? 8 : 4;
  auto al = [](size_t b) { return (b + 15) & ~size_t(15); };
  size_t b = 0;
  for (int l = bl; l <= lc; ++l) {
    const Level &L = mg->lev[l];
    const size_t nnz = L.h_rowptr[L.n];
    b += al((L.n + 1) * 4) + al(size_t(L.n) * 4) + al(nnz * 4) + al(nnz * ss * T) + al(size_t(L.n) * ss * T) +
         2 * al(L.n);
    b += al(L.lower.ptr.size() * 4) + al(L.upper.ptr.size() * 4) + 2 * al(size_t(L.n) * 4);
    if (smo == 2 && l > bl) b += 2 * (al((L.n + 1) * 4) + al(nnz * 4) + al(nnz * ss * T)) + al(size_t(L.n) * ss * T);
    if (l > bl)
      b += al((L.n + 1) * 4) + al(L.P.nnz * 4) + al(L.P.nnz * T) + al((mg->lev[l - 1].n + 1) * 4) +
           al(L.R.nnz * 4) + al(L.R.nnz * T);
    b += 3 * al(size_t(L.n) * s * T);
  }
  const size_t N = size_t(mg->lev[bl].n) * s;
  b += al(N * N * 8);
  return (long long)b;
}

template <class KERN>
static int set_smem(KERN kern, int bytes) {
  static thread_local std::map<void *, int> smem_set;
  if (smem_set[(void *)kern] < bytes) {
    GMG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    smem_set[(void *)kern] = bytes;
  }
  return 0;
}

int k_coarse_cycle(gmg_mg *mg, int prec, const CoarseCfg &cfg, gmg_vec *c, gmg_vec *b, gmg_vec *t) {
  (void)t;
  int err = 0;
  CachedImage *ci = get_image(mg, cfg.bl, cfg.lc, prec, cfg.smoother, &err);
  if (!ci) return 1;
  const int s = mg->lev[cfg.bl].s;
  int unit = 1;
  for (int r = 0; r < s; ++r)
    if (cfg.damp[r] != 1.0) unit = 0;
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  lc.stream = mg->stream;
  lc.attrs = attr;
  lc.numAttrs = mg->opts.disable_pdl ? 0 : 1;
  lc.dynamicSmemBytes = ci->smem;
  if (ci->batched) {
    BCall call{};
    call.nu1 = cfg.nu1;
    call.nu2 = cfg.nu2;
    call.unit_damp = unit;
    call.bl = cfg.bl;
    for (int r = 0; r < GMG_MAX_S; ++r) {
      call.damp[r] = cfg.damp[r];
      call.cdamp[r] = cfg.cdamp[r];
      call.abslimit[r] = cfg.abslimit[r];
    }
    for (int k = 0; k <= cfg.lc - cfg.bl; ++k) {
      call.gb[k] = b->lev[cfg.bl + k];
      call.gc[k] = c->lev[cfg.bl + k];
    }
    void (*kern)(const SArgs *, const BCall) = nullptr;
#define PICK(TT, SS)                                                               \
  if (s == SS) {                                                                   \
    if (cfg.smoother == 0) kern = coarse_cycle_batched_kernel<TT, SS, 0>;          \
    else if (cfg.smoother == 1) kern = coarse_cycle_batched_kernel<TT, SS, 1>;     \
    else kern = coarse_cycle_batched_kernel<TT, SS, 2>;                            \
  }
    if (prec == GMG_PREC_FP64) { PICK(double, 1) PICK(double, 2) PICK(double, 3) }
    else { PICK(float, 1) PICK(float, 2) PICK(float, 3) }
#undef PICK
    GMG_CHECK(kern, "block size %d not compiled", s);
    if (set_smem(kern, ci->smem)) return 1;
    lc.gridDim = dim3(ci->ninst);
    lc.blockDim = dim3(BBLK);
    GMG_CUDA(cudaLaunchKernelEx(&lc, kern, (const SArgs *)ci->dev_args, call));
    mg->launches++;
    return 0;
  }
  SArgs a = ci->args;
  if (!cfg.narrow) a.narrow = 0;
  a.nu1 = cfg.nu1;
  a.nu2 = cfg.nu2;
  a.unit_damp = unit;
  for (int r = 0; r < GMG_MAX_S; ++r) {
    a.damp[r] = cfg.damp[r];
    a.cdamp[r] = cfg.cdamp[r];
    a.abslimit[r] = cfg.abslimit[r];
  }
  for (int k = 0; k < a.nl; ++k) {
    a.L[k].gb = b->lev[cfg.bl + k];
    a.L[k].gc = c->lev[cfg.bl + k];
  }
  void (*kern)(const SArgs) = nullptr;
#define PICK(TT, SS)                                                     \
  if (s == SS) {                                                         \
    if (cfg.smoother == 0) kern = coarse_cycle_kernel<TT, SS, 0>;        \
    else if (cfg.smoother == 1) kern = coarse_cycle_kernel<TT, SS, 1>;   \
    else kern = coarse_cycle_kernel<TT, SS, 2>;                          \
  }
  if (prec == GMG_PREC_FP64) { PICK(double, 1) PICK(double, 2) PICK(double, 3) }
  else { PICK(float, 1) PICK(float, 2) PICK(float, 3) }
#undef PICK
  GMG_CHECK(kern, "block size %d not compiled", s);
  if (set_smem(kern, a.smem_bytes)) return 1;
  lc.gridDim = dim3(1);
  lc.blockDim = dim3(CBLK);
  GMG_CUDA(cudaLaunchKernelEx(&lc, kern, a));
  mg->launches++;
  return 0;
}

}  // namespace gmg
