// ILU(0) decomposition on the device: l_ilubthdecomp (np/algebra/ugiter.cc:
// 2252-2625) without threshold and rest vector, as ILUPreProcess runs it
// (np/procs/iter.cc:5444) on a copy of the level matrix, in the level's
// processing order, with the beta modification of the diagonal.
//
// UG eliminates row by row ("right-looking"): pivot i inverts its diagonal
// block D_i, then for every active row j > i of its pattern forms the pivot
// L_ji = A_ji D_i^{-1} and subtracts L_ji A_ik from every pattern entry
// (j, k), k > i, adding |L_ji A_ik| to row j's beta row sum where (j, k) is
// missing.  Entry (j, k) so receives the updates of the pivots i in
// ascending order.  Here each row j gathers them itself ("IKJ"): it walks
// its strictly lower entries (j, i) in ascending i, every row i being final,
// which applies the same updates in the same order -- the factors are the
// host elimination's bit for bit (all products and sums rounded separately,
// never contracted into FMAs).  Rows of one wavefront of the level's forward
// schedule (level sets of the lower triangle) have no lower entry inside the
// wavefront, so a launch per wavefront factors them all at once; the
// pattern must be structurally symmetric, as UG's MATRIX pairs are.
//
// The combined factor array (processing-order CSR of the level: D_i^{-1} on
// the diagonal, L below, U above, inactive rows untouched) is then split
// into the sweep's arrays: the unit lower factor, the strict upper factor and
// the inverted diagonal blocks, FP64 and (if built) FP32.
#include <climits>

#include "gmg_internal.h"

namespace gmg {

namespace {

constexpr int ILU_BLK = 128;

#define LAUNCH_CHECK(mg)                                                                \
  do {                                                                                  \
    (mg)->launches++;                                                                   \
    cudaError_t e_ = cudaGetLastError();                                                \
    if (e_ != cudaSuccess) {                                                            \
      set_error("%s:%d kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      return 1;                                                                         \
    }                                                                                   \
  } while (0)

struct IluBeta {
  double b[GMG_MAX_S];
};

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// the inverse of an S x S block (the host's invert_block: 1/m, Cramer for
// 2 x 2, Gauss-Jordan with partial pivoting above); false if singular
template <int S>
__device__ bool invert_small(const double *m, double *inv) {
  if (S == 1) {
    if (m[0] == 0.0) return false;
    inv[0] = __ddiv_rn(1.0, m[0]);
    return true;
  }
  if (S == 2) {
    const double det = sub(mul(m[0], m[3]), mul(m[1], m[2]));
    if (det == 0.0) return false;
    const double id = __ddiv_rn(1.0, det);
    inv[0] = mul(m[3], id); inv[1] = mul(-m[1], id); inv[2] = mul(-m[2], id); inv[3] = mul(m[0], id);
    return true;
  }
  double a[S * S];
  for (int q = 0; q < S * S; ++q) { a[q] = m[q]; inv[q] = 0.0; }
  for (int q = 0; q < S; ++q) inv[q * S + q] = 1.0;
  for (int c = 0; c < S; ++c) {
    int p = c;
    for (int r = c + 1; r < S; ++r)
      if (fabs(a[r * S + c]) > fabs(a[p * S + c])) p = r;
    if (a[p * S + c] == 0.0) return false;
    if (p != c)
      for (int k = 0; k < S; ++k) {
        double t = a[p * S + k]; a[p * S + k] = a[c * S + k]; a[c * S + k] = t;
        t = inv[p * S + k]; inv[p * S + k] = inv[c * S + k]; inv[c * S + k] = t;
      }
    const double d = __ddiv_rn(1.0, a[c * S + c]);
    for (int k = 0; k < S; ++k) { a[c * S + k] = mul(a[c * S + k], d); inv[c * S + k] = mul(inv[c * S + k], d); }
    for (int r = 0; r < S; ++r) {
      if (r == c) continue;
      const double f = a[r * S + c];
      if (f == 0.0) continue;
      for (int k = 0; k < S; ++k) {
        a[r * S + k] = sub(a[r * S + k], mul(f, a[c * S + k]));
        inv[r * S + k] = sub(inv[r * S + k], mul(f, inv[c * S + k]));
      }
    }
  }
  return true;
}

// position of column k in row j (entries jb..je-1), -1 if absent
__device__ __forceinline__ int find_col(const int *__restrict__ col, int jb, int je, int k) {
  for (int e = jb; e < je; ++e)
    if (col[e] == k) return e;
  return -1;
}

// one wavefront: every active row j of it eliminates its lower entries in
// ascending column order, then inverts its diagonal block.  A failed
// inversion records the smallest failing row in *fail.
template <int S>
__global__ void __launch_bounds__(ILU_BLK) ilu_factor_wave_kernel(const int *__restrict__ rows, int nr,
                                                                const int *__restrict__ rowptr,
                                                                const int *__restrict__ col,
                                                                const uint8_t *__restrict__ flags,
                                                                const int *__restrict__ lsptr,
                                                                const int *__restrict__ lsort, double *lu,
                                                                IluBeta beta, int *fail) {
  constexpr int SS = S * S;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nr) return;
  const int j = rows[t];
  if (!(flags[j] & F_ACTIVE)) return;
  const int jb = rowptr[j], je = rowptr[j + 1];
  double *djj = lu + (size_t)jb * SS;
  for (int q = lsptr[j]; q < lsptr[j + 1]; ++q) {
    const int kji = lsort[q];
    const int i = col[kji];
    if (!(flags[i] & F_ACTIVE)) continue;
    const int ib = rowptr[i], ie = rowptr[i + 1];
    const double *inv = lu + (size_t)ib * SS;  // D_i^{-1}: row i is final
    double *piv = lu + (size_t)kji * SS;
    if (S == 1) {
      const double pivot = mul(piv[0], inv[0]);
      piv[0] = pivot;
      if (pivot == 0.0) continue;
      for (int kik = ib + 1; kik < ie; ++kik) {
        const int k = col[kik];
        if (!((flags[k] & F_ACTIVE) && k > i)) continue;
        const double prod = mul(pivot, lu[kik]);
        const int kjk = find_col(col, jb, je, k);
        if (kjk >= 0) lu[kjk] = sub(lu[kjk], prod);
        else djj[0] = add(djj[0], mul(beta.b[0], fabs(prod)));
      }
      continue;
    }
    double pm[SS];
    bool zero = true;
#pragma unroll
    for (int r = 0; r < S; ++r)
#pragma unroll
      for (int c = 0; c < S; ++c) {
        double sum = 0.0;
#pragma unroll
        for (int w = 0; w < S; ++w) sum = add(sum, mul(piv[r * S + w], inv[w * S + c]));
        pm[r * S + c] = sum;
        if (sum != 0.0) zero = false;
      }
#pragma unroll
    for (int w = 0; w < SS; ++w) piv[w] = pm[w];
    if (zero) continue;
    double rowsum[S];
#pragma unroll
    for (int r = 0; r < S; ++r) rowsum[r] = 0.0;
    for (int kik = ib + 1; kik < ie; ++kik) {
      const int k = col[kik];
      if (!((flags[k] & F_ACTIVE) && i < k)) continue;
      const double *elm = lu + (size_t)kik * SS;
      double cor[SS];
      bool cz = true;
#pragma unroll
      for (int r = 0; r < S; ++r)
#pragma unroll
        for (int c = 0; c < S; ++c) {
          double sum = 0.0;
#pragma unroll
          for (int w = 0; w < S; ++w) sum = add(sum, mul(pm[r * S + w], elm[w * S + c]));
          cor[r * S + c] = sum;
          if (sum != 0.0) cz = false;
        }
      if (cz) continue;
      const int kjk = find_col(col, jb, je, k);
      if (kjk >= 0) {
        double *mat = lu + (size_t)kjk * SS;
#pragma unroll
        for (int w = 0; w < SS; ++w) mat[w] = sub(mat[w], cor[w]);
      } else {
#pragma unroll
        for (int r = 0; r < S; ++r)
#pragma unroll
          for (int c = 0; c < S; ++c) rowsum[r] = add(rowsum[r], fabs(cor[r * S + c]));
      }
    }
#pragma unroll
    for (int r = 0; r < S; ++r)
#pragma unroll
      for (int c = 0; c < S; ++c) djj[r * S + c] = mul(djj[r * S + c], add(1.0, mul(beta.b[c], rowsum[c])));
  }
  // StoreInverse: the diagonal block becomes its inverse
  bool ok;
  if (S == 1) {
    const double d = djj[0];
    ok = !(fabs(d) < 2.220446049250313e-16 * 10 * 1e-20);
    if (ok) djj[0] = __ddiv_rn(1.0, d);
  } else {
    double inv[SS];
    ok = invert_small<S>(djj, inv);
    if (ok)
#pragma unroll
      for (int w = 0; w < SS; ++w) djj[w] = inv[w];
  }
  if (!ok) atomicMin(fail, j);
}

// the factors into the sweep's arrays: per row, entries in CSR order
template <int S>
__global__ void __launch_bounds__(ILU_BLK) ilu_split_kernel(int n, const int *__restrict__ rowptr,
                                                          const int *__restrict__ col,
                                                          const uint8_t *__restrict__ flags,
                                                          const double *__restrict__ lu,
                                                          const int *__restrict__ lrp, const int *__restrict__ urp,
                                                          double *lv, double *uv, double *ud, float *lv32,
                                                          float *uv32, float *ud32) {
  constexpr int SS = S * S;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool act = flags[i] & F_ACTIVE;
  int lp = lrp[i], up = urp[i];
  if (!act) {
#pragma unroll
    for (int w = 0; w < SS; ++w) {
      ud[(size_t)i * SS + w] = 0.0;
      if (ud32) ud32[(size_t)i * SS + w] = 0.0f;
    }
    return;
  }
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const int j = col[k];
    const double *src = lu + (size_t)k * SS;
    double *dst;
    float *dst32;
    if (j == i) {
      dst = ud + (size_t)i * SS;
      dst32 = ud32 ? ud32 + (size_t)i * SS : nullptr;
    } else if (!(flags[j] & F_ACTIVE)) {
      continue;
    } else if (j < i) {
      dst = lv + (size_t)lp * SS;
      dst32 = lv32 ? lv32 + (size_t)lp * SS : nullptr;
      ++lp;
    } else {
      dst = uv + (size_t)up * SS;
      dst32 = uv32 ? uv32 + (size_t)up * SS : nullptr;
      ++up;
    }
#pragma unroll
    for (int w = 0; w < SS; ++w) {
      dst[w] = src[w];
      if (dst32) dst32[w] = float(src[w]);
    }
  }
}

template <int S>
int ilu_factor_s(gmg_mg *mg, Level &L, const double *beta, const IluDev &D, int *failed_row) {
  IluBeta b;
  for (int r = 0; r < GMG_MAX_S; ++r) b.b[r] = beta[r];
  const int init = INT_MAX;
  GMG_CUDA(cudaMemcpyAsync(D.fail, &init, sizeof(int), cudaMemcpyHostToDevice, mg->stream));
  GMG_CUDA(cudaMemcpyAsync(D.lu, L.A.v64, sizeof(double) * L.nnzb * S * S, cudaMemcpyDeviceToDevice, mg->stream));
  for (int w = 0; w < L.lower.nwave(); ++w) {
    const int r0 = L.lower.ptr[w], nr = L.lower.ptr[w + 1] - r0;
    if (nr <= 0) continue;
    ilu_factor_wave_kernel<S><<<(nr + ILU_BLK - 1) / ILU_BLK, ILU_BLK, 0, mg->stream>>>(
        L.lower.rows + r0, nr, L.A.rowptr, L.A.col, L.flags, D.lsptr, D.lsort, D.lu, b, D.fail);
    LAUNCH_CHECK(mg);
  }
  int fail = INT_MAX;
  GMG_CUDA(cudaMemcpyAsync(&fail, D.fail, sizeof(int), cudaMemcpyDeviceToHost, mg->stream));
  GMG_CUDA(cudaStreamSynchronize(mg->stream));
  if (fail != INT_MAX) {
    *failed_row = fail;
    return 0;
  }
  ilu_split_kernel<S><<<(L.n + ILU_BLK - 1) / ILU_BLK, ILU_BLK, 0, mg->stream>>>(
      L.n, L.A.rowptr, L.A.col, L.flags, D.lu, L.L.rowptr, L.U.rowptr, L.L.v64, L.U.v64, L.udinv64, L.L.v32,
      L.U.v32, L.udinv32);
  LAUNCH_CHECK(mg);
  return 0;
}

}  // namespace

int k_ilu_factor(gmg_mg *mg, Level &L, const double *beta, const IluDev &D, int *failed_row) {
  *failed_row = -1;
  if (L.n == 0) return 0;
  switch (L.s) {
    case 1: return ilu_factor_s<1>(mg, L, beta, D, failed_row);
    case 2: return ilu_factor_s<2>(mg, L, beta, D, failed_row);
    case 3: return ilu_factor_s<3>(mg, L, beta, D, failed_row);
    default: set_error("ILU: block size %d not compiled", L.s); return 1;
  }
}

}  // namespace gmg
