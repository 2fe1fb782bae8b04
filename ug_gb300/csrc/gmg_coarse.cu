// Fused coarse-grid cycle: the lmgc recursion (gamma = 1) over the small
// levels bl..lc run by ONE thread-block cluster in a single launch.
//
// Below a few tens of thousands of unknowns a level's kernels are far
// shorter than a launch, so a V-cycle there is launch-latency bound (each
// level needs ~40 dependent kernels per visit).  Here every phase of
// Lmgc (np/procs/iter.cc:7741) -- smoothing step, defect update, dadd,
// restriction, coarse reset, base solve, interpolation -- is a
// cluster-strided loop over the level's rows, separated from the next
// phase by the hardware cluster barrier (barrier.cluster, release/acquire
// at cluster scope) instead of a kernel boundary.  Data written inside the
// kernel (b, c, t) is read through L2 (ld.global.cg) so that no SM reads a
// stale L1 line written by another SM of the cluster; matrix data is
// read-only and uses the read-only path.  The arithmetic of each phase is
// that of the per-level kernels in gmg_kernels.cu.
#include <cooperative_groups.h>

#include "gmg_internal.h"
#include "gmg_np.h"

namespace gmg {

namespace {

constexpr int MAXCL = 12;
constexpr int CBLK = 512;

template <class T>
struct CLev {
  int n, all_active;
  const int *rowptr, *col;
  const T *val, *dinv;
  const uint8_t *flags, *skip;
  int nwave, nuwave;
  const int *wptr, *wrows, *uptr, *urows;
  const int *lrow, *lcol, *urow, *ucol;
  const T *lval, *uval, *udinv;
  const int *prow, *pcol, *rrow, *rcol;  // P (rows: this level), R (rows: level below)
  const T *pw, *rw;
  T *c, *b, *t;
};

template <class T>
struct CArgs {
  int nl;  // levels in the fused range; L[0] is the base level
  int nu1, nu2, unit_damp;
  T damp[GMG_MAX_S], cdamp[GMG_MAX_S];
  const double *ainv;
  double abslimit[GMG_MAX_S];
  CLev<T> L[MAXCL];
};

__device__ __forceinline__ void cluster_sync() {
  __threadfence();
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

template <class T>
__device__ __forceinline__ T ldv(const T *p) { return __ldcg(p); }

struct Team {
  int tid, nth, rank;
};

// x -= A y ; acc += y (dmatmul_minus + dadd)
template <class T, int S>
__device__ void c_spmv(const CLev<T> &L, T *x, const T *y, T *acc, const Team &tm) {
  for (int i = tm.tid; i < L.n; i += tm.nth) {
    T s[S];
#pragma unroll
    for (int r = 0; r < S; ++r) s[r] = T(0);
    const int k1 = __ldg(L.rowptr + i + 1);
    for (int k = __ldg(L.rowptr + i); k < k1; ++k) {
      const int j = __ldg(L.col + k);
      const T *m = L.val + (size_t)k * S * S;
#pragma unroll
      for (int r = 0; r < S; ++r)
#pragma unroll
        for (int c = 0; c < S; ++c) s[r] = fma(__ldg(m + r * S + c), ldv(y + (size_t)j * S + c), s[r]);
    }
#pragma unroll
    for (int r = 0; r < S; ++r) {
      x[(size_t)i * S + r] = ldv(x + (size_t)i * S + r) - s[r];
      if (acc) acc[(size_t)i * S + r] = ldv(acc + (size_t)i * S + r) + ldv(y + (size_t)i * S + r);
    }
  }
}

// t = damp * D^{-1} b (l_jac + dscalx)
template <class T, int S>
__device__ void c_jac(const CLev<T> &L, const CArgs<T> &a, const Team &tm) {
  for (int i = tm.tid; i < L.n; i += tm.nth) {
    if (!L.all_active && !(L.flags[i] & F_ACTIVE)) {
#pragma unroll
      for (int r = 0; r < S; ++r) L.t[(size_t)i * S + r] = T(0);
      continue;
    }
    T bv[S];
#pragma unroll
    for (int c = 0; c < S; ++c) bv[c] = ldv(L.b + (size_t)i * S + c);
#pragma unroll
    for (int r = 0; r < S; ++r) {
      T v = T(0);
#pragma unroll
      for (int c = 0; c < S; ++c) v = fma(__ldg(L.dinv + (size_t)i * S * S + r * S + c), bv[c], v);
      L.t[(size_t)i * S + r] = v * a.damp[r];
    }
  }
}

// (D+L) t = b over the wavefronts, L = entries to rows earlier in processing order (l_lgs)
template <class T, int S>
__device__ void c_gs(const CLev<T> &L, const Team &tm) {
  for (int w = 0; w < L.nwave; ++w) {
    const int r0 = __ldg(L.wptr + w), r1 = __ldg(L.wptr + w + 1);
    for (int q = r0 + tm.tid; q < r1; q += tm.nth) {
      const int i = __ldg(L.wrows + q);
      if (!L.all_active && !(L.flags[i] & F_ACTIVE)) {
#pragma unroll
        for (int r = 0; r < S; ++r) L.t[(size_t)i * S + r] = T(0);
        continue;
      }
      T s[S];
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = ldv(L.b + (size_t)i * S + r);
      const int k1 = __ldg(L.rowptr + i + 1);
      for (int k = __ldg(L.rowptr + i) + 1; k < k1; ++k) {
        const int j = __ldg(L.col + k);
        if (j >= i) continue;
        const T *m = L.val + (size_t)k * S * S;
#pragma unroll
        for (int r = 0; r < S; ++r)
#pragma unroll
          for (int c = 0; c < S; ++c) s[r] = fma(-__ldg(m + r * S + c), ldv(L.t + (size_t)j * S + c), s[r]);
      }
#pragma unroll
      for (int r = 0; r < S; ++r) {
        T v = T(0);
#pragma unroll
        for (int c = 0; c < S; ++c) v = fma(__ldg(L.dinv + (size_t)i * S * S + r * S + c), s[c], v);
        L.t[(size_t)i * S + r] = v;
      }
    }
    cluster_sync();
  }
}

// L U t = b (l_luiter): forward waves with the unit lower factor, backward with U and D^{-1}
template <class T, int S>
__device__ void c_ilu(const CLev<T> &L, const Team &tm) {
  for (int w = 0; w < L.nwave; ++w) {
    const int r0 = __ldg(L.wptr + w), r1 = __ldg(L.wptr + w + 1);
    for (int q = r0 + tm.tid; q < r1; q += tm.nth) {
      const int i = __ldg(L.wrows + q);
      const bool act = L.all_active || (L.flags[i] & F_ACTIVE);
      T s[S];
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = act ? ldv(L.b + (size_t)i * S + r) : T(0);
      if (act) {
        const int k1 = __ldg(L.lrow + i + 1);
        for (int k = __ldg(L.lrow + i); k < k1; ++k) {
          const int j = __ldg(L.lcol + k);
          const T *m = L.lval + (size_t)k * S * S;
#pragma unroll
          for (int r = 0; r < S; ++r)
#pragma unroll
            for (int c = 0; c < S; ++c) s[r] = fma(-__ldg(m + r * S + c), ldv(L.t + (size_t)j * S + c), s[r]);
        }
      }
#pragma unroll
      for (int r = 0; r < S; ++r) L.t[(size_t)i * S + r] = s[r];
    }
    cluster_sync();
  }
  for (int w = 0; w < L.nuwave; ++w) {
    const int r0 = __ldg(L.uptr + w), r1 = __ldg(L.uptr + w + 1);
    for (int q = r0 + tm.tid; q < r1; q += tm.nth) {
      const int i = __ldg(L.urows + q);
      if (!L.all_active && !(L.flags[i] & F_ACTIVE)) continue;
      T s[S];
#pragma unroll
      for (int r = 0; r < S; ++r) s[r] = ldv(L.t + (size_t)i * S + r);
      const int k1 = __ldg(L.urow + i + 1);
      for (int k = __ldg(L.urow + i); k < k1; ++k) {
        const int j = __ldg(L.ucol + k);
        const T *m = L.uval + (size_t)k * S * S;
#pragma unroll
        for (int r = 0; r < S; ++r)
#pragma unroll
          for (int c = 0; c < S; ++c) s[r] = fma(-__ldg(m + r * S + c), ldv(L.t + (size_t)j * S + c), s[r]);
      }
#pragma unroll
      for (int r = 0; r < S; ++r) {
        T v = T(0);
#pragma unroll
        for (int c = 0; c < S; ++c) v = fma(__ldg(L.udinv + (size_t)i * S * S + r * S + c), s[c], v);
        L.t[(size_t)i * S + r] = v;
      }
    }
    cluster_sync();
  }
}

template <class T, int S>
__device__ void c_scale(const CLev<T> &L, const CArgs<T> &a, const Team &tm) {
  for (int i = tm.tid; i < L.n; i += tm.nth)
#pragma unroll
    for (int r = 0; r < S; ++r) L.t[(size_t)i * S + r] = ldv(L.t + (size_t)i * S + r) * a.damp[r];
}

// one smoothing step of Smoother (iter.cc:817) followed by lmgc's dadd(c, t)
template <class T, int S, int SMO>
__device__ void c_smooth(const CLev<T> &L, const CArgs<T> &a, const Team &tm) {
  if (SMO == 0) {
    c_jac<T, S>(L, a, tm);
    cluster_sync();
  } else {
    if (SMO == 1) c_gs<T, S>(L, tm);
    else c_ilu<T, S>(L, tm);
    if (!a.unit_damp) {
      c_scale<T, S>(L, a, tm);
      cluster_sync();
    }
  }
  c_spmv<T, S>(L, L.b, L.t, L.c, tm);
  cluster_sync();
}

// StandardRestrict into the level below, fused with lmgc's dset(c_{l-1}, 0)
template <class T, int S>
__device__ void c_restrict(const CLev<T> &F, const CLev<T> &Cl, const Team &tm) {
  for (int c = tm.tid; c < Cl.n; c += tm.nth) {
    const bool reset = Cl.flags[c] & F_RESET;
    const int sk = Cl.skip[c];
    T acc[S];
#pragma unroll
    for (int r = 0; r < S; ++r) acc[r] = reset ? T(0) : ldv(Cl.b + (size_t)c * S + r);
    const int k1 = __ldg(F.rrow + c + 1);
    for (int k = __ldg(F.rrow + c); k < k1; ++k) {
      const int f = __ldg(F.rcol + k);
      const T w = __ldg(F.rw + k);
#pragma unroll
      for (int r = 0; r < S; ++r) acc[r] = fma(w, ldv(F.b + (size_t)f * S + r), acc[r]);
    }
#pragma unroll
    for (int r = 0; r < S; ++r) {
      if (!(sk & (1 << r))) Cl.b[(size_t)c * S + r] = acc[r];
      else if (reset) Cl.b[(size_t)c * S + r] = T(0);
      Cl.c[(size_t)c * S + r] = T(0);
    }
  }
}

// StandardInterpolateCorrection into t, fused with lmgc's dadd(c, t)
template <class T, int S>
__device__ void c_interp(const CLev<T> &F, const CLev<T> &Cl, const CArgs<T> &a, const Team &tm) {
  for (int f = tm.tid; f < F.n; f += tm.nth) {
    const int sk = F.skip[f];
    T v[S];
#pragma unroll
    for (int r = 0; r < S; ++r) v[r] = T(0);
    if (sk != (1 << S) - 1) {
      const int k1 = __ldg(F.prow + f + 1);
      for (int k = __ldg(F.prow + f); k < k1; ++k) {
        const int c = __ldg(F.pcol + k);
        const T w = __ldg(F.pw + k);
#pragma unroll
        for (int r = 0; r < S; ++r) v[r] = fma(w * a.cdamp[r], ldv(Cl.c + (size_t)c * S + r), v[r]);
      }
#pragma unroll
      for (int r = 0; r < S; ++r)
        if (sk & (1 << r)) v[r] = T(0);
    }
#pragma unroll
    for (int r = 0; r < S; ++r) {
      F.t[(size_t)f * S + r] = v[r];
      F.c[(size_t)f * S + r] = ldv(F.c + (size_t)f * S + r) + v[r];
    }
  }
}

// base solver `ls $m 1 $I ex` on the cluster's first CTA
template <class T, int S>
__device__ void c_base(const CLev<T> &B, const CArgs<T> &a) {
  __shared__ double red[S][CBLK / 32];
  __shared__ int skip;
  double acc[S];
#pragma unroll
  for (int r = 0; r < S; ++r) acc[r] = 0.0;
  for (int i = threadIdx.x; i < B.n; i += blockDim.x)
#pragma unroll
    for (int r = 0; r < S; ++r) {
      double v = double(ldv(B.b + (size_t)i * S + r));
      acc[r] += v * v;
    }
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
      for (int w = 0; w < CBLK / 32; ++w) v += red[r][w];
      if (fabs(sqrt(v)) >= fabs(a.abslimit[r])) below = 0;
    }
    skip = below;
  }
  __syncthreads();
  if (skip) return;
  const int N = B.n * S;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double v = 0.0;
    for (int j = 0; j < N; ++j) v = fma(a.ainv[(size_t)i * N + j], double(ldv(B.b + j)), v);
    B.t[i] = T(v);
  }
  __syncthreads();
  Team one{int(threadIdx.x), int(blockDim.x), 0};
  c_spmv<T, S>(B, B.b, B.t, B.c, one);
}

template <class T, int S, int SMO>
__global__ void __launch_bounds__(CBLK, 1) coarse_cycle_kernel(const __grid_constant__ CArgs<T> a) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  Team tm;
  tm.rank = int(cl.block_rank());
  tm.nth = int(cl.num_blocks()) * blockDim.x;
  tm.tid = tm.rank * blockDim.x + threadIdx.x;
  // down: pre-smoothing and restriction, from the top of the fused range
  for (int k = a.nl - 1; k >= 1; --k) {
    for (int it = 0; it < a.nu1; ++it) c_smooth<T, S, SMO>(a.L[k], a, tm);
    c_restrict<T, S>(a.L[k], a.L[k - 1], tm);
    cluster_sync();
  }
  if (tm.rank == 0) c_base<T, S>(a.L[0], a);
  cluster_sync();
  // up: interpolation, coarse-grid correction, post-smoothing
  for (int k = 1; k < a.nl; ++k) {
    c_interp<T, S>(a.L[k], a.L[k - 1], a, tm);
    cluster_sync();
    c_spmv<T, S>(a.L[k], a.L[k].b, a.L[k].t, nullptr, tm);
    cluster_sync();
    for (int it = 0; it < a.nu2; ++it) c_smooth<T, S, SMO>(a.L[k], a, tm);
  }
}

template <class T>
const T *pick(const double *d, const float *f);
template <>
const double *pick<double>(const double *d, const float *) { return d; }
template <>
const float *pick<float>(const double *, const float *f) { return f; }

template <class T>
int fill_args(gmg_mg *mg, const CoarseCfg &cfg, gmg_vec *c, gmg_vec *b, gmg_vec *t, CArgs<T> &a) {
  a.nl = cfg.lc - cfg.bl + 1;
  GMG_CHECK(a.nl >= 1 && a.nl <= MAXCL, "fused coarse cycle: %d levels (max %d)", a.nl, MAXCL);
  a.nu1 = cfg.nu1;
  a.nu2 = cfg.nu2;
  a.unit_damp = 1;
  const int s = mg->lev[cfg.bl].s;
  for (int r = 0; r < GMG_MAX_S; ++r) {
    a.damp[r] = T(cfg.damp[r]);
    a.cdamp[r] = T(cfg.cdamp[r]);
    a.abslimit[r] = cfg.abslimit[r];
    if (r < s && cfg.damp[r] != 1.0) a.unit_damp = 0;
  }
  const Level &B = mg->lev[cfg.bl];
  GMG_CHECK(B.ainv, "base level inverse not computed (ex PreProcess)");
  a.ainv = B.ainv;
  for (int k = 0; k < a.nl; ++k) {
    const Level &L = mg->lev[cfg.bl + k];
    CLev<T> &d = a.L[k];
    d.n = L.n;
    d.all_active = L.all_active;
    d.rowptr = L.A.rowptr; d.col = L.A.col;
    d.val = pick<T>(L.A.v64, L.A.v32);
    d.dinv = pick<T>(L.dinv64, L.dinv32);
    GMG_CHECK(d.val && d.dinv, "fused coarse cycle: precision copy missing");
    d.flags = L.flags; d.skip = L.skip;
    d.nwave = L.lower.nwave(); d.wptr = L.lower.ptr_dev; d.wrows = L.lower.rows;
    d.nuwave = L.upper.nwave(); d.uptr = L.upper.ptr_dev; d.urows = L.upper.rows;
    d.lrow = L.L.rowptr; d.lcol = L.L.col; d.lval = pick<T>(L.L.v64, L.L.v32);
    d.urow = L.U.rowptr; d.ucol = L.U.col; d.uval = pick<T>(L.U.v64, L.U.v32);
    d.udinv = pick<T>(L.udinv64, L.udinv32);
    if (cfg.smoother == 2 && k > 0) GMG_CHECK(L.ilu_ready && d.lval && d.uval, "ILU factors missing on level %d", cfg.bl + k);
    d.prow = L.P.rowptr; d.pcol = L.P.col; d.pw = pick<T>(L.P.v64, L.P.v32);
    d.rrow = L.R.rowptr; d.rcol = L.R.col; d.rw = pick<T>(L.R.v64, L.R.v32);
    d.c = (T *)c->lev[cfg.bl + k];
    d.b = (T *)b->lev[cfg.bl + k];
    d.t = (T *)t->lev[cfg.bl + k];
  }
  return 0;
}

template <class T, int S, int SMO>
int launch(gmg_mg *mg, const CArgs<T> &a, int want_cluster) {
  auto kern = coarse_cycle_kernel<T, S, SMO>;
  // the cluster size is chosen once per kernel variant, outside any stream
  // capture: the largest power of two <= want_cluster that fits
  static int chosen[2][4][3][6] = {};
  int wi = 0;
  while ((1 << wi) < want_cluster && wi < 5) ++wi;
  int &csz = chosen[sizeof(T) == 8 ? 0 : 1][S][SMO][wi];
  if (!csz) {
    GMG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    for (int c = 1 << wi; c >= 1; c /= 2) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = c;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3(c);
      cfg.blockDim = dim3(CBLK);
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters >= 1) {
        csz = c;
        break;
      }
      cudaGetLastError();
    }
    GMG_CHECK(csz, "fused coarse cycle: no cluster size fits");
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csz;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(csz);
  cfg.blockDim = dim3(CBLK);
  cfg.stream = mg->stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  GMG_CUDA(cudaLaunchKernelEx(&cfg, kern, a));
  mg->launches++;
  return 0;
}

template <class T>
int dispatch(gmg_mg *mg, const CoarseCfg &cfg, gmg_vec *c, gmg_vec *b, gmg_vec *t) {
  CArgs<T> a;
  if (fill_args<T>(mg, cfg, c, b, t, a)) return 1;
  const int s = mg->lev[cfg.bl].s;
#define L3(SS)                                                                  \
  if (s == SS) {                                                                \
    if (cfg.smoother == 0) return launch<T, SS, 0>(mg, a, cfg.cluster);         \
    if (cfg.smoother == 1) return launch<T, SS, 1>(mg, a, cfg.cluster);         \
    return launch<T, SS, 2>(mg, a, cfg.cluster);                                \
  }
  L3(1) L3(2) L3(3)
#undef L3
  set_error("block size %d not compiled", s);
  return 1;
}

}  // namespace

int k_coarse_cycle(gmg_mg *mg, int prec, const CoarseCfg &cfg, gmg_vec *c, gmg_vec *b, gmg_vec *t) {
  if (prec == GMG_PREC_FP64) return dispatch<double>(mg, cfg, c, b, t);
  return dispatch<float>(mg, cfg, c, b, t);
}

}  // namespace gmg
