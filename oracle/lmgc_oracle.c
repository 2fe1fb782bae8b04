/* lmgc_oracle.c -- sequential C restatement of UG 3.12.1's lmgc path.
 * TEST INFRASTRUCTURE ONLY (see lmgc_oracle.h).  Each function names the
 * reference routine whose arithmetic it restates. */
#include "lmgc_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ACTIVE_CLASS 3 /* gm/algebra.h: vectors the smoothers update */
#define NEWDEF_CLASS 2 /* gm/algebra.h: vectors carrying a new defect */

/* SolveSmallBlock, np/algebra/block.cc:104-224: n=1 division, n=2 Cramer
 * with the inverted determinant, n=3 the reference's elimination formula,
 * larger n Gaussian elimination with partial pivoting. */
static int solve_small(int n, double *sol, const double *m, const double *rhs) {
  if (n == 1) { sol[0] = rhs[0] / m[0]; return 0; }
  if (n == 2) {
    double det = m[0] * m[3] - m[1] * m[2];
    if (det == 0.0) return 1;
    det = 1.0 / det;
    sol[0] = (rhs[0] * m[3] - rhs[1] * m[1]) * det;
    sol[1] = (rhs[1] * m[0] - rhs[0] * m[2]) * det;
    return 0;
  }
  if (n == 3) {
    double M3div0 = m[3] / m[0], M6div0 = m[6] / m[0];
    double aux = (m[7] - M6div0 * m[1]) / (m[4] - M3div0 * m[1]);
    sol[2] = (rhs[2] - M6div0 * rhs[0] - aux * (rhs[1] - M3div0 * rhs[0])) /
             (m[8] - M6div0 * m[2] - aux * (m[5] - M3div0 * m[2]));
    sol[1] = (rhs[1] - m[3] / m[0] * rhs[0] - (m[5] - M3div0 * m[2]) * sol[2]) / (m[4] - M3div0 * m[1]);
    sol[0] = (rhs[0] - m[1] * sol[1] - m[2] * sol[2]) / m[0];
    return 0;
  }
  double a[ORC_MAX_S * ORC_MAX_S], b[ORC_MAX_S];
  memcpy(a, m, sizeof(double) * n * n);
  memcpy(b, rhs, sizeof(double) * n);
  for (int i = 0; i < n; ++i) {
    int p = i;
    for (int k = i + 1; k < n; ++k) if (fabs(a[k * n + i]) > fabs(a[p * n + i])) p = k;
    if (a[p * n + i] == 0.0) return 1;
    if (p != i) {
      for (int k = 0; k < n; ++k) { double t = a[i * n + k]; a[i * n + k] = a[p * n + k]; a[p * n + k] = t; }
      double t = b[i]; b[i] = b[p]; b[p] = t;
    }
    for (int k = i + 1; k < n; ++k) {
      double f = a[k * n + i] / a[i * n + i];
      for (int j = i; j < n; ++j) a[k * n + j] -= f * a[i * n + j];
      b[k] -= f * b[i];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= a[i * n + j] * sol[j];
    sol[i] = s / a[i * n + i];
  }
  return 0;
}

/* InvertSmallBlock, block.cc:272-330 (n=1,2 closed form; larger n by
 * solving against the unit vectors). */
static int invert_small(int n, const double *m, double *inv) {
  if (n == 1) {
    if (fabs(m[0]) < 1e-25) return 1;
    inv[0] = 1.0 / m[0];
    return 0;
  }
  if (n == 2) {
    double det = m[0] * m[3] - m[1] * m[2];
    if (fabs(det) < 1e-25) return 1;
    double id = 1.0 / det;
    inv[0] = m[3] * id; inv[1] = -m[1] * id; inv[2] = -m[2] * id; inv[3] = m[0] * id;
    return 0;
  }
  if (n == 3) {
    double det = m[0] * m[4] * m[8] + m[1] * m[5] * m[6] + m[2] * m[3] * m[7] - m[2] * m[4] * m[6] -
                 m[0] * m[5] * m[7] - m[1] * m[3] * m[8];
    if (fabs(det) < 1e-25) return 1;
    double id = 1.0 / det;
    inv[0] = (m[4] * m[8] - m[5] * m[7]) * id;
    inv[3] = (-m[3] * m[8] + m[5] * m[6]) * id;
    inv[6] = (m[3] * m[7] - m[4] * m[6]) * id;
    inv[1] = (-m[1] * m[8] + m[2] * m[7]) * id;
    inv[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    inv[7] = (-m[0] * m[7] + m[1] * m[6]) * id;
    inv[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    inv[5] = (-m[0] * m[5] + m[2] * m[3]) * id;
    inv[8] = (m[0] * m[4] - m[1] * m[3]) * id;
    return 0;
  }
  for (int c = 0; c < n; ++c) {
    double e[ORC_MAX_S] = {0}, x[ORC_MAX_S];
    e[c] = 1.0;
    if (solve_small(n, x, m, e)) return 1;
    for (int r = 0; r < n; ++r) inv[r * n + c] = x[r];
  }
  return 0;
}

/* dmatmul_minus, np/algebra/ugblas.cc:3997 (templates matfunc.ct /
 * matloop.ct, MATMUL_rc macros ugblas.h:161-340): per row the products of
 * all row entries (diagonal first) are summed, then subtracted once. */
void orc_matmul_minus(const orc_level *L, double *x, const double *y) {
  const int s = L->s, ss = s * s;
  for (int i = 0; i < L->n; ++i) {
    double acc[ORC_MAX_S] = {0};
    for (int k = L->rowptr[i]; k < L->rowptr[i + 1]; ++k) {
      const double *m = L->val + (size_t)k * ss;
      const double *w = y + (size_t)L->col[k] * s;
      for (int r = 0; r < s; ++r) {
        double t = 0.0;
        for (int c = 0; c < s; ++c) t += m[r * s + c] * w[c];
        acc[r] += t;
      }
    }
    for (int r = 0; r < s; ++r) x[(size_t)i * s + r] -= acc[r];
  }
}

/* l_jac, np/algebra/ugiter.cc:271-356: v = D^{-1} d on ACTIVE vectors,
 * zero elsewhere. */
int orc_jac(const orc_level *L, double *v, const double *d) {
  const int s = L->s, ss = s * s;
  for (int i = 0; i < L->n; ++i) {
    double *vi = v + (size_t)i * s;
    if (L->vclass[i] < ACTIVE_CLASS) { for (int r = 0; r < s; ++r) vi[r] = 0.0; continue; }
    const double *D = L->val + (size_t)L->rowptr[i] * ss;
    if (s == 1) vi[0] = d[i] / D[0];
    else if (solve_small(s, vi, D, d + (size_t)i * s)) return -(i + 1);
  }
  return 0;
}

/* l_lgs, ugiter.cc:412-612: forward solve of (D+L) v = d in list order,
 * L = entries to ACTIVE vectors earlier in the list. */
int orc_lgs(const orc_level *L, double *v, const double *d) {
  const int s = L->s, ss = s * s;
  for (int i = 0; i < L->n; ++i) {
    double *vi = v + (size_t)i * s;
    if (L->vclass[i] < ACTIVE_CLASS) { for (int r = 0; r < s; ++r) vi[r] = 0.0; continue; }
    const int k0 = L->rowptr[i];
    if (s == 1) {
      double sum = 0.0;
      for (int k = k0 + 1; k < L->rowptr[i + 1]; ++k) {
        int j = L->col[k];
        if (j < i && L->vclass[j] >= ACTIVE_CLASS) sum += L->val[k] * v[j];
      }
      vi[0] = (d[i] - sum) / L->val[k0];
    } else {
      double rhs[ORC_MAX_S], acc[ORC_MAX_S] = {0};
      for (int r = 0; r < s; ++r) rhs[r] = d[(size_t)i * s + r];
      for (int k = k0 + 1; k < L->rowptr[i + 1]; ++k) {
        int j = L->col[k];
        if (!(j < i && L->vclass[j] >= ACTIVE_CLASS)) continue;
        const double *m = L->val + (size_t)k * ss, *w = v + (size_t)j * s;
        for (int r = 0; r < s; ++r) {
          double t = 0.0;
          for (int c = 0; c < s; ++c) t += m[r * s + c] * w[c];
          acc[r] += t;
        }
      }
      for (int r = 0; r < s; ++r) rhs[r] -= acc[r];
      if (solve_small(s, vi, L->val + (size_t)k0 * ss, rhs)) return -(i + 1);
    }
  }
  return 0;
}

static int find_entry(const orc_level *L, int row, int col) {
  for (int k = L->rowptr[row]; k < L->rowptr[row + 1]; ++k)
    if (L->col[k] == col) return k;
  return -1;
}

/* l_ilubthdecomp, ugiter.cc:2252-2625, without threshold / rest vector
 * (as called by ILUPreProcess, np/procs/iter.cc:5444): in-place ILU(0) in
 * list order.  Row i's diagonal block is replaced by its inverse
 * (StoreInverse), each (j,i) below it by the pivot L_ji = A_ji D_i^{-1},
 * and the pattern entries (j,k), k>i, are updated.  Off-pattern fill is
 * dropped; beta adds it back to the diagonal (scalar: beta*|fill|,
 * blocks: the diagonal's columns scaled by 1+beta*rowsum). */
int orc_ilu_decomp(const orc_level *L, double *lu, const double *beta) {
  const int s = L->s, ss = s * s, n = L->n;
  memcpy(lu, L->val, sizeof(double) * (size_t)L->rowptr[n] * ss);
  for (int i = 0; i < n; ++i) {
    if (L->vclass[i] < ACTIVE_CLASS) continue;
    const int kd = L->rowptr[i];
    if (s == 1) {
      double diag = lu[kd];
      if (fabs(diag) < DBL_EPSILON * 10 * 1e-20) return -(i + 1);
      double invdiag = 1.0 / diag;
      lu[kd] = invdiag;
      for (int kij = kd + 1; kij < L->rowptr[i + 1]; ++kij) {
        int j = L->col[kij];
        if (!(L->vclass[j] >= ACTIVE_CLASS && j > i)) continue;
        int kji = find_entry(L, j, i);
        double pivot = lu[kji] * invdiag;
        lu[kji] = pivot;
        if (pivot == 0.0) continue;
        for (int kik = kd + 1; kik < L->rowptr[i + 1]; ++kik) {
          int k = L->col[kik];
          if (!(L->vclass[k] >= ACTIVE_CLASS && k > i)) continue;
          int kjk = find_entry(L, j, k);
          if (kjk >= 0) lu[kjk] -= pivot * lu[kik];
          else if (beta) lu[L->rowptr[j]] += beta[0] * fabs(pivot * lu[kik]);
        }
      }
    } else {
      double inv[ORC_MAX_S * ORC_MAX_S];
      if (invert_small(s, lu + (size_t)kd * ss, inv)) return -(i + 1);
      memcpy(lu + (size_t)kd * ss, inv, sizeof(double) * ss);
      for (int kij = kd + 1; kij < L->rowptr[i + 1]; ++kij) {
        int j = L->col[kij];
        if (!(L->vclass[j] >= ACTIVE_CLASS && i < j)) continue;
        double rowsum[ORC_MAX_S] = {0};
        int kji = find_entry(L, j, i);
        double *piv = lu + (size_t)kji * ss, pm[ORC_MAX_S * ORC_MAX_S];
        int zero = 1;
        for (int r = 0; r < s; ++r)
          for (int c = 0; c < s; ++c) {
            double sum = 0.0;
            for (int q = 0; q < s; ++q) sum += piv[r * s + q] * inv[q * s + c];
            pm[r * s + c] = sum;
            if (sum != 0.0) zero = 0;
          }
        memcpy(piv, pm, sizeof(double) * ss);
        if (zero) continue;
        for (int kik = kd + 1; kik < L->rowptr[i + 1]; ++kik) {
          int k = L->col[kik];
          if (!(L->vclass[k] >= ACTIVE_CLASS && i < k)) continue;
          const double *elm = lu + (size_t)kik * ss;
          double cor[ORC_MAX_S * ORC_MAX_S];
          int cz = 1;
          for (int r = 0; r < s; ++r)
            for (int c = 0; c < s; ++c) {
              double sum = 0.0;
              for (int q = 0; q < s; ++q) sum += pm[r * s + q] * elm[q * s + c];
              cor[r * s + c] = sum;
              if (sum != 0.0) cz = 0;
            }
          if (cz) continue;
          int kjk = find_entry(L, j, k);
          if (kjk >= 0) {
            double *mat = lu + (size_t)kjk * ss;
            for (int q = 0; q < ss; ++q) mat[q] -= cor[q];
          } else {
            for (int r = 0; r < s; ++r)
              for (int c = 0; c < s; ++c) rowsum[r] += fabs(cor[r * s + c]);
          }
        }
        if (!beta) continue;
        double *djj = lu + (size_t)L->rowptr[j] * ss;
        for (int r = 0; r < s; ++r)
          for (int c = 0; c < s; ++c) djj[r * s + c] *= 1.0 + beta[c] * rowsum[c];
      }
    }
  }
  return 0;
}

/* l_luiter, ugiter.cc:4444-4796: forward solve with the unit lower factor
 * in list order, then backward solve with the upper factor in reverse list
 * order, multiplying by the stored inverse diagonal. */
int orc_luiter(const orc_level *L, const double *lu, double *v, const double *d) {
  const int s = L->s, ss = s * s, n = L->n;
  for (int i = 0; i < n; ++i) {
    double *vi = v + (size_t)i * s;
    if (L->vclass[i] < ACTIVE_CLASS) { for (int r = 0; r < s; ++r) vi[r] = 0.0; continue; }
    double acc[ORC_MAX_S] = {0};
    for (int k = L->rowptr[i] + 1; k < L->rowptr[i + 1]; ++k) {
      int j = L->col[k];
      if (!(j < i && L->vclass[j] >= ACTIVE_CLASS)) continue;
      const double *m = lu + (size_t)k * ss, *w = v + (size_t)j * s;
      if (s == 1) { acc[0] += m[0] * w[0]; continue; }
      for (int r = 0; r < s; ++r) {
        double t = 0.0;
        for (int c = 0; c < s; ++c) t += m[r * s + c] * w[c];
        acc[r] += t;
      }
    }
    for (int r = 0; r < s; ++r) vi[r] = d[(size_t)i * s + r] - acc[r];
  }
  for (int i = n - 1; i >= 0; --i) {
    if (L->vclass[i] < ACTIVE_CLASS) continue;
    double *vi = v + (size_t)i * s;
    double acc[ORC_MAX_S] = {0};
    for (int k = L->rowptr[i] + 1; k < L->rowptr[i + 1]; ++k) {
      int j = L->col[k];
      if (!(j > i && L->vclass[j] >= ACTIVE_CLASS)) continue;
      const double *m = lu + (size_t)k * ss, *w = v + (size_t)j * s;
      if (s == 1) { acc[0] += m[0] * w[0]; continue; }
      for (int r = 0; r < s; ++r) {
        double t = 0.0;
        for (int c = 0; c < s; ++c) t += m[r * s + c] * w[c];
        acc[r] += t;
      }
    }
    const double *dinv = lu + (size_t)L->rowptr[i] * ss;
    if (s == 1) { vi[0] = (vi[0] - acc[0]) * dinv[0]; continue; }
    double rhs[ORC_MAX_S];
    for (int r = 0; r < s; ++r) rhs[r] = vi[r] - acc[r];
    for (int r = 0; r < s; ++r) {
      double sum = 0.0;
      for (int c = 0; c < s; ++c) sum += dinv[r * s + c] * rhs[c];
      vi[r] = sum;
    }
  }
  return 0;
}

/* dnrm2x, ugblas.cc:3156: per-component Euclidean norms, summed in list
 * order over the vectors with NEW_DEFECT (VCLASS >= 2), which is the
 * ON_SURFACE set of the top level of a uniformly refined hierarchy. */
void orc_nrm2x(const orc_level *L, const double *x, double *out) {
  const int s = L->s;
  for (int r = 0; r < s; ++r) out[r] = 0.0;
  for (int i = 0; i < L->n; ++i) {
    if (L->vclass[i] < NEWDEF_CLASS) continue;
    for (int r = 0; r < s; ++r) { double v = x[(size_t)i * s + r]; out[r] += v * v; }
  }
  for (int r = 0; r < s; ++r) out[r] = sqrt(out[r]);
}

/* StandardRestrictNodeVector, np/algebra/transgrid.cc:117-232: reset the
 * coarse vectors with VNCLASS >= NEWDEF_CLASS, then every fine vector with
 * VCLASS >= NEWDEF_CLASS adds weight*damp*value to its coarse parents,
 * except into components the coarse VECSKIP marks. */
void orc_restrict(const orc_level *fine, const orc_level *coarse, double *to, const double *from,
                  const double *damp) {
  const int s = fine->s;
  for (int c = 0; c < coarse->n; ++c)
    if (coarse->vnclass[c] >= NEWDEF_CLASS)
      for (int r = 0; r < s; ++r) to[(size_t)c * s + r] = 0.0;
  for (int f = 0; f < fine->n; ++f) {
    if (fine->vclass[f] < NEWDEF_CLASS) continue;
    double sv[ORC_MAX_S];
    for (int r = 0; r < s; ++r) sv[r] = damp[r] * from[(size_t)f * s + r];
    for (int k = fine->prowptr[f]; k < fine->prowptr[f + 1]; ++k) {
      int c = fine->pcol[k];
      int sk = coarse->skip[c];
      for (int r = 0; r < s; ++r)
        if (!(sk & (1 << r))) to[(size_t)c * s + r] += fine->pw[k] * sv[r];
    }
  }
}

/* StandardIntCorNodeVector, transgrid.cc:235-347: reset the fine vector,
 * then every fine vector not skipped in all components takes
 * sum_i weight_i*damp*coarse_i in each component its VECSKIP leaves free. */
void orc_interpolate(const orc_level *fine, double *to, const double *from, const double *damp) {
  const int s = fine->s;
  memset(to, 0, sizeof(double) * (size_t)fine->n * s);
  for (int f = 0; f < fine->n; ++f) {
    int sk = fine->skip[f];
    if (sk == (1 << s) - 1) continue;
    for (int r = 0; r < s; ++r) {
      if (sk & (1 << r)) continue;
      double acc = 0.0;
      for (int k = fine->prowptr[f]; k < fine->prowptr[f + 1]; ++k)
        acc += fine->pw[k] * damp[r] * from[(size_t)fine->pcol[k] * s + r];
      to[(size_t)f * s + r] = acc;
    }
  }
}

/* RestrictByMatrix_General, np/algebra/transgrid.cc:1113-1247 (flag 0): the
 * coarse vectors with VNCLASS >= NEWDEF_CLASS are reset; every fine vector
 * with VCLASS >= NEWDEF_CLASS adds block * d to each coarse vector of its
 * interpolation matrix, in the components that coarse vector's VECSKIP
 * leaves free (block row i times the fine vector, summed over j first);
 * then the reset coarse vectors are scaled by damp if any damp != 1.  (UG's
 * CRITBIT filter is never set on these hierarchies.) */
void orc_restrict_imat(const orc_level *fine, const orc_imat *M, const orc_level *coarse, double *to,
                       const double *from, const double *damp) {
  const int s = fine->s, ss = s * s;
  for (int c = 0; c < coarse->n; ++c)
    if (coarse->vnclass[c] >= NEWDEF_CLASS)
      for (int r = 0; r < s; ++r) to[(size_t)c * s + r] = 0.0;
  for (int f = 0; f < fine->n; ++f) {
    if (fine->vclass[f] < NEWDEF_CLASS) continue;
    const double *v = from + (size_t)f * s;
    for (int k = M->rowptr[f]; k < M->rowptr[f + 1]; ++k) {
      const int c = M->col[k], sk = coarse->skip[c];
      const double *m = M->val + (size_t)k * ss;
      for (int i = 0; i < s; ++i) {
        if (sk & (1 << i)) continue;
        double sum = 0.0;
        for (int j = 0; j < s; ++j) sum += m[i * s + j] * v[j];
        to[(size_t)c * s + i] += sum;
      }
    }
  }
  int scale = 0;
  for (int r = 0; r < s; ++r) scale |= damp[r] != 1.0;
  if (scale)
    for (int c = 0; c < coarse->n; ++c)
      if (coarse->vnclass[c] >= NEWDEF_CLASS)
        for (int r = 0; r < s; ++r) to[(size_t)c * s + r] *= damp[r];
}

/* InterpolateCorrectionByMatrix_General, transgrid.cc:1292-1386 (flag 0):
 * the fine level is reset; every fine vector takes, in each component its
 * VECSKIP leaves free, the transposed blocks of its interpolation matrix
 * times the coarse vectors (sum over the coarse components first, coarse
 * vectors in list order); then every fine vector is scaled by damp if any
 * damp != 1. */
void orc_interpolate_imat(const orc_level *fine, const orc_imat *M, double *to, const double *from,
                          const double *damp) {
  const int s = fine->s, ss = s * s;
  memset(to, 0, sizeof(double) * (size_t)fine->n * s);
  for (int f = 0; f < fine->n; ++f) {
    const int sk = fine->skip[f];
    for (int k = M->rowptr[f]; k < M->rowptr[f + 1]; ++k) {
      const double *m = M->val + (size_t)k * ss, *w = from + (size_t)M->col[k] * s;
      for (int i = 0; i < s; ++i) {
        if (sk & (1 << i)) continue;
        double sum = 0.0;
        for (int j = 0; j < s; ++j) sum += m[j * s + i] * w[j];
        to[(size_t)f * s + i] += sum;
      }
    }
  }
  int scale = 0;
  for (int r = 0; r < s; ++r) scale |= damp[r] != 1.0;
  if (scale)
    for (int f = 0; f < fine->n; ++f)
      for (int r = 0; r < s; ++r) to[(size_t)f * s + r] *= damp[r];
}

/* InterpolateNewVectorsByMatrix, transgrid.cc:1425-1490: every fine vector
 * with VNEW set takes the product of its interpolation-matrix row with the
 * coarse vector.  One component per vector (the scalar descriptor branch,
 * 1436-1453): only vectors with VECSKIP 0, each entry added to x directly.
 * Blocks (1456-1488): VECSKIP not consulted, per entry the block's
 * transposed product (m[j s + i], as InterpolateCorrectionByMatrix) summed
 * into one value and then added.  The other fine vectors keep theirs. */
void orc_interpolate_new_imat(const orc_level *fine, const orc_imat *M, const int *vnew, double *x_fine,
                              const double *x_coarse) {
  const int s = fine->s, ss = s * s;
  for (int f = 0; f < fine->n; ++f) {
    if (!vnew[f]) continue;
    double *v = x_fine + (size_t)f * s;
    if (s == 1) {
      if (fine->skip[f]) continue;
      v[0] = 0.0;
      for (int k = M->rowptr[f]; k < M->rowptr[f + 1]; ++k) v[0] += M->val[k] * x_coarse[M->col[k]];
      continue;
    }
    for (int i = 0; i < s; ++i) v[i] = 0.0;
    for (int k = M->rowptr[f]; k < M->rowptr[f + 1]; ++k) {
      const double *m = M->val + (size_t)k * ss, *w = x_coarse + (size_t)M->col[k] * s;
      for (int i = 0; i < s; ++i) {
        double sum = 0.0;
        for (int j = 0; j < s; ++j) sum += m[j * s + i] * w[j];
        v[i] += sum;
      }
    }
  }
}

/* StandardIntNewNodeVector, np/algebra/transgrid.cc:354-430: every fine
 * vector with VNEW set takes the coarse values through its transfer row (a
 * corner copy, or the father element's shape functions GNs), every
 * component, VECSKIP not consulted; the other fine vectors keep theirs. */
void orc_interpolate_new(const orc_level *fine, const int *vnew, double *x_fine, const double *x_coarse) {
  const int s = fine->s;
  for (int f = 0; f < fine->n; ++f) {
    if (!vnew[f]) continue;
    for (int r = 0; r < s; ++r) {
      double acc = 0.0;
      for (int k = fine->prowptr[f]; k < fine->prowptr[f + 1]; ++k)
        acc += fine->pw[k] * x_coarse[(size_t)fine->pcol[k] * s + r];
      x_fine[(size_t)f * s + r] = acc;
    }
  }
}

/* StandardProject, transgrid.cc:655-700 (node vectors): a coarse vector
 * whose node has a son node takes the son's values.  The son is the fine
 * corner copy, the fine vector whose transfer row is the single weight 1. */
void orc_project(const orc_level *fine, double *x_coarse, const double *x_fine) {
  const int s = fine->s;
  for (int f = 0; f < fine->n; ++f) {
    const int k = fine->prowptr[f];
    if (fine->prowptr[f + 1] - k != 1 || fine->pw[k] != 1.0) continue;
    for (int r = 0; r < s; ++r) x_coarse[(size_t)fine->pcol[k] * s + r] = x_fine[(size_t)f * s + r];
  }
}

/* ---------------------------------------------------------------- solver */
typedef struct {
  const orc_mg *mg;
  double **c, **t, **b, **lu; /* per level */
  int *own_b;                 /* b of the level allocated here (not the caller's) */
  double *base_lu;            /* dense LU of the base level (no pivoting) */
  int base_n;
} orc_ws;

/* ex base solver, np/procs/iter.cc:8685-9068 with the band LU of
 * gm/evm.cc (EXDecomposeMatrixDOUBLE / EXApplyLUDOUBLE): LU without
 * pivoting in list order; the dense matrix here is the band with full width. */
static int base_factor(orc_ws *w, const orc_level *L) {
  const int s = L->s, n = L->n * s;
  w->base_n = n;
  w->base_lu = (double *)calloc((size_t)n * n, sizeof(double));
  if (!w->base_lu) return -1;
  double *M = w->base_lu;
  for (int i = 0; i < L->n; ++i)
    for (int k = L->rowptr[i]; k < L->rowptr[i + 1]; ++k)
      for (int r = 0; r < s; ++r)
        for (int c = 0; c < s; ++c) M[(size_t)(i * s + r) * n + L->col[k] * s + c] = L->val[(size_t)k * s * s + r * s + c];
  for (int i = 0; i < n - 1; ++i) {
    double d = M[(size_t)i * n + i];
    if (d == 0.0) return -1;
    for (int j = i + 1; j < n; ++j) {
      double f = M[(size_t)j * n + i] / d;
      M[(size_t)j * n + i] = f;
      for (int k = i + 1; k < n; ++k) M[(size_t)j * n + k] -= f * M[(size_t)i * n + k];
    }
  }
  return 0;
}

static void base_apply(const orc_ws *w, double *vec) {
  const int n = w->base_n;
  const double *M = w->base_lu;
  for (int i = 1; i < n; ++i)
    for (int j = 0; j < i; ++j) vec[i] -= M[(size_t)i * n + j] * vec[j];
  for (int i = n - 1; i >= 0; --i) {
    for (int j = i + 1; j < n; ++j) vec[i] -= M[(size_t)i * n + j] * vec[j];
    vec[i] /= M[(size_t)i * n + i];
  }
}

/* Smoother, iter.cc:817-842: t = Step(b); t *= damp; b -= A t. */
static int smooth(orc_ws *w, int l, double *t, double *b) {
  const orc_mg *mg = w->mg;
  const orc_level *L = &mg->lev[l];
  const int s = L->s;
  int rc;
  if (mg->smoother == ORC_JAC) rc = orc_jac(L, t, b);
  else if (mg->smoother == ORC_GS) rc = orc_lgs(L, t, b);
  else rc = orc_luiter(L, w->lu[l], t, b);
  if (rc) return rc;
  for (int i = 0; i < L->n; ++i)
    for (int r = 0; r < s; ++r) t[(size_t)i * s + r] *= mg->damp[r];
  orc_matmul_minus(L, b, t);
  return 0;
}

static void vadd(double *x, const double *y, size_t n) { for (size_t i = 0; i < n; ++i) x[i] += y[i]; }

/* Lmgc, iter.cc:7741-7949. */
static int lmgc(orc_ws *w, int l) {
  const orc_mg *mg = w->mg;
  const orc_level *L = &mg->lev[l];
  const size_t len = (size_t)L->n * L->s;
  double *c = w->c[l], *b = w->b[l], *t = w->t[l];
  int rc;
  if (l <= mg->baselevel) {
    /* base ls with $m 1 and the ex iteration: c += A^{-1} b; b -= A (A^{-1} b),
     * skipped when the defect is already below the base abslimit */
    double nb[ORC_MAX_S];
    orc_nrm2x(L, b, nb);
    int below = 1;
    for (int r = 0; r < L->s; ++r)
      if (fabs(nb[r]) >= fabs(mg->base_abslimit[r])) below = 0;
    if (below) return 0;
    memcpy(t, b, sizeof(double) * len);
    base_apply(w, t);
    orc_matmul_minus(L, b, t);
    vadd(c, t, len);
    return 0;
  }
  for (int i = 0; i < mg->nu1; ++i) {
    if ((rc = smooth(w, l, t, b))) return rc;
    vadd(c, t, len);
  }
  const orc_level *Lc = &mg->lev[l - 1];
  double one[ORC_MAX_S];
  for (int r = 0; r < ORC_MAX_S; ++r) one[r] = 1.0;
  if (mg->imat)
    orc_restrict_imat(L, &mg->imat[l], Lc, w->b[l - 1], b, one);
  else
    orc_restrict(L, Lc, w->b[l - 1], b, one);
  memset(w->c[l - 1], 0, sizeof(double) * (size_t)Lc->n * Lc->s);
  for (int g = 0; g < mg->gamma; ++g)
    if ((rc = lmgc(w, l - 1))) return rc;
  if (mg->imat)
    orc_interpolate_imat(L, &mg->imat[l], t, w->c[l - 1], mg->cdamp);
  else
    orc_interpolate(L, t, w->c[l - 1], mg->cdamp);
  vadd(c, t, len);
  orc_matmul_minus(L, b, t);
  for (int i = 0; i < mg->nu2; ++i) {
    if ((rc = smooth(w, l, t, b))) return rc;
    vadd(c, t, len);
  }
  return 0;
}

/* sc_cmp, np/udm/npscan.cc:1027-1057: 1 iff every |x_i| < |y_i|. */
static int sc_cmp(const double *x, const double *y, int s) {
  for (int i = 0; i < s; ++i)
    if (fabs(x[i]) >= fabs(y[i])) return 0;
  return 1;
}

/* LinearSolver, np/procs/ls.cc:637-749, preceded by LinearDefect (562) and
 * LinearResiduum (577); LSUpdate (869) adds c on levels baselevel..top. */
/* the lmgc workspace of levels bl..top; b of a level is the caller's where
 * bl_caller[l] is given (always for the top level), else allocated here */
static int ws_init_levels(orc_ws *w, const orc_mg *mg, double *const *b_caller) {
  const int top = mg->nlevels - 1;
  const int s = mg->lev[top].s;
  const int bl = mg->baselevel < top ? mg->baselevel : top;
  memset(w, 0, sizeof *w);
  w->mg = mg;
  w->c = (double **)calloc(mg->nlevels, sizeof(double *));
  w->t = (double **)calloc(mg->nlevels, sizeof(double *));
  w->b = (double **)calloc(mg->nlevels, sizeof(double *));
  w->lu = (double **)calloc(mg->nlevels, sizeof(double *));
  w->own_b = (int *)calloc(mg->nlevels, sizeof(int));
  for (int l = bl; l <= top; ++l) {
    size_t len = (size_t)mg->lev[l].n * s;
    w->c[l] = (double *)calloc(len, sizeof(double));
    w->t[l] = (double *)calloc(len, sizeof(double));
    w->own_b[l] = b_caller[l] == NULL;
    w->b[l] = w->own_b[l] ? (double *)calloc(len, sizeof(double)) : b_caller[l];
    if (mg->smoother == ORC_ILU && l > bl) {
      const orc_level *L = &mg->lev[l];
      int rc;
      w->lu[l] = (double *)malloc(sizeof(double) * (size_t)L->rowptr[L->n] * s * s);
      if ((rc = orc_ilu_decomp(L, w->lu[l], mg->beta))) return rc;
    }
  }
  if (base_factor(w, &mg->lev[bl])) return -1000000;
  return 0;
}

/* the workspace of a solve whose defect lives on the top level only */
static int ws_init(orc_ws *w, const orc_mg *mg, double *b) {
  double *bc[64] = {0};
  if (mg->nlevels > 64) return -1;
  bc[mg->nlevels - 1] = b;
  return ws_init_levels(w, mg, bc);
}

static void ws_free(orc_ws *w) {
  const orc_mg *mg = w->mg;
  const int top = mg->nlevels - 1;
  const int bl = mg->baselevel < top ? mg->baselevel : top;
  for (int l = bl; l <= top; ++l) {
    free(w->c[l]); free(w->t[l]); free(w->lu[l]);
    if (w->own_b && w->own_b[l]) free(w->b[l]);
  }
  free(w->c); free(w->t); free(w->b); free(w->lu); free(w->base_lu); free(w->own_b);
}

/* dmatmul, ugblas.cc:3782: x = A y, per row the products summed, then assigned */
static void matmul(const orc_level *L, double *x, const double *y) {
  const int s = L->s, ss = s * s;
  for (int i = 0; i < L->n; ++i) {
    double acc[ORC_MAX_S] = {0};
    for (int k = L->rowptr[i]; k < L->rowptr[i + 1]; ++k) {
      const double *m = L->val + (size_t)k * ss;
      const double *w = y + (size_t)L->col[k] * s;
      for (int r = 0; r < s; ++r) {
        double t = 0.0;
        for (int c = 0; c < s; ++c) t += m[r * s + c] * w[c];
        acc[r] += t;
      }
    }
    for (int r = 0; r < s; ++r) x[(size_t)i * s + r] = acc[r];
  }
}

/* ddot ON_SURFACE, ugblas.cc:3104: one sum over the NEW_DEFECT vectors of the
 * top level, components in order, vectors in list order */
static double ddot(const orc_level *L, const double *x, const double *y) {
  const int s = L->s;
  double sum = 0.0;
  for (int i = 0; i < L->n; ++i) {
    if (L->vclass[i] < NEWDEF_CLASS) continue;
    for (int r = 0; r < s; ++r) sum += x[(size_t)i * s + r] * y[(size_t)i * s + r];
  }
  return sum;
}

int orc_cg_solve(const orc_mg *mg, double *x, double *b, const double *red, const double *abslimit, int maxit,
                 double *hist, int *converged) {
  const int top = mg->nlevels - 1;
  const int s = mg->lev[top].s;
  const orc_level *T = &mg->lev[top];
  const size_t len = (size_t)T->n * s;
  orc_ws w;
  int rc = ws_init(&w, mg, b), it = 0;
  double *p = (double *)calloc(len, sizeof(double)), *t = (double *)calloc(len, sizeof(double));
  *converged = 0;
  if (rc) goto done;
  {
    double first[ORC_MAX_S], last[ORC_MAX_S], reach[ORC_MAX_S], rho = 1.0; /* CGPrepare, ls.cc:976 */
    orc_matmul_minus(T, b, x);
    orc_nrm2x(T, b, first);
    if (hist) for (int r = 0; r < s; ++r) hist[r] = first[r];
    for (int r = 0; r < s; ++r) { reach[r] = first[r] * red[r]; if (reach[r] == 0.0) reach[r] = red[r]; }
    *converged = sc_cmp(first, abslimit, s);
    for (it = 0; it < maxit; ++it) {
      if (*converged) break;
      double *c = w.c[top];
      memset(c, 0, sizeof(double) * len);
      if ((rc = lmgc(&w, top))) goto done;
      /* CGUpdate, ls.cc:989-1064 */
      matmul(T, t, c);
      vadd(b, t, len);
      double lambda = ddot(T, c, b);
      const double f = lambda / rho;
      for (size_t i = 0; i < len; ++i) p[i] *= f;
      rho = lambda;
      vadd(p, c, len);
      matmul(T, t, p);
      lambda = ddot(T, t, p);
      if (lambda == 0.0) { rc = -2000000; goto done; }
      const double a = rho / lambda, na = -rho / lambda;
      for (size_t i = 0; i < len; ++i) x[i] += a * p[i];
      for (size_t i = 0; i < len; ++i) b[i] += na * t[i];
      orc_nrm2x(T, b, last);
      if (hist) for (int r = 0; r < s; ++r) hist[(size_t)(it + 1) * s + r] = last[r];
      if (sc_cmp(last, abslimit, s) || sc_cmp(last, reach, s)) { *converged = 1; ++it; break; }
    }
  }
done:
  free(p); free(t);
  ws_free(&w);
  return rc ? rc : it;
}

/* ddotw ON_SURFACE, ugblas.cc:3023 (weights 1): per-component sums over the
 * NEW_DEFECT vectors of the top level, then added component by component */
static double ddotw(const orc_level *L, const double *x, const double *y) {
  const int s = L->s;
  double a[ORC_MAX_S] = {0};
  for (int i = 0; i < L->n; ++i) {
    if (L->vclass[i] < NEWDEF_CLASS) continue;
    for (int r = 0; r < s; ++r) a[r] += x[(size_t)i * s + r] * y[(size_t)i * s + r];
  }
  double sum = 0.0;
  for (int r = 0; r < s; ++r) sum += 1.0 * a[r];
  return sum;
}

/* sc_eq, npscan.cc:1095 */
static int sc_eq(const double *x, const double *y, double ac, int s) {
  for (int i = 0; i < s; ++i)
    if (x[i] < 0.0 || y[i] < 0.0 || fabs(x[i] - y[i]) > ac * sqrt(x[i] * y[i])) return 0;
  return 1;
}

/* the preconditioner q = lmgc(d) on a scratch copy of d (Iter updates its defect) */
static int precond(orc_ws *w, int top, double *q, const double *d, size_t len) {
  double *bt = w->b[top];
  memcpy(bt, d, sizeof(double) * len);
  memset(w->c[top], 0, sizeof(double) * len);
  int rc = lmgc(w, top);
  memcpy(q, w->c[top], sizeof(double) * len);
  return rc;
}

int orc_bcgs_solve(const orc_mg *mg, double *x, double *b, const double *red, const double *abslimit, int maxit,
                   double *hist, int *converged) {
  const int top = mg->nlevels - 1;
  const int s = mg->lev[top].s;
  const orc_level *T = &mg->lev[top];
  const size_t len = (size_t)T->n * s;
  orc_ws w;
  double *scratch = (double *)calloc(len, sizeof(double));
  int rc = ws_init(&w, mg, scratch), iters = 0;
  double *r = (double *)calloc(len, sizeof(double)), *p = (double *)calloc(len, sizeof(double)),
         *v = (double *)calloc(len, sizeof(double)), *sv = (double *)calloc(len, sizeof(double)),
         *t = (double *)calloc(len, sizeof(double)), *q = (double *)calloc(len, sizeof(double));
  *converged = 0;
  if (rc) goto done;
  {
    double first[ORC_MAX_S], last[ORC_MAX_S], reach[ORC_MAX_S], old[ORC_MAX_S];
    double alpha = 0.0, rho_new = 0.0, beta = 0.0, tt = 0.0, rho = 0.0, omega = 0.0;
    int restart = 1, eq_count = 0, nh = 0;
    for (int k = 0; k < s; ++k) old[k] = -1.0; /* BCGSPreProcess, ls.cc:1831 */
    orc_matmul_minus(T, b, x);
    orc_nrm2x(T, b, first);
    if (hist) for (int k = 0; k < s; ++k) hist[k] = first[k];
    for (int k = 0; k < s; ++k) { reach[k] = first[k] * red[k]; if (reach[k] == 0.0) reach[k] = red[k]; }
    *converged = sc_cmp(first, abslimit, s);
    /* BCGSSolver, ls.cc:1864-2062 (no restart index, weights 1) */
    for (int i = 0; i < maxit; ++i) {
      if (*converged) break;
      if (restart) {
        memset(p, 0, sizeof(double) * len);
        memset(v, 0, sizeof(double) * len);
        memcpy(r, b, sizeof(double) * len);
        alpha = rho = omega = 1.0;
        restart = 0;
      }
      rho_new = ddotw(T, b, r);
      if (rho != 0.0 && omega != 0.0) beta = rho_new * alpha / rho / omega;
      for (size_t k = 0; k < len; ++k) p[k] *= beta;
      vadd(p, b, len);
      { const double a = -beta * omega; for (size_t k = 0; k < len; ++k) p[k] += a * v[k]; }
      if ((rc = precond(&w, top, q, p, len))) goto done;
      matmul(T, v, q);
      alpha = ddotw(T, v, r);
      if (alpha != 0.0) alpha = rho_new / alpha;
      for (size_t k = 0; k < len; ++k) x[k] += alpha * q[k];
      ++iters;
      memcpy(sv, b, sizeof(double) * len);
      { const double a = -alpha; for (size_t k = 0; k < len; ++k) sv[k] += a * v[k]; }
      orc_nrm2x(T, sv, last);
      ++nh;
      if (hist) for (int k = 0; k < s; ++k) hist[(size_t)nh * s + k] = last[k];
      if (sc_cmp(last, abslimit, s) || sc_cmp(last, reach, s)) {
        memcpy(b, sv, sizeof(double) * len);
        *converged = 1;
        break;
      }
      if ((rc = precond(&w, top, q, sv, len))) goto done;
      matmul(T, t, q);
      tt = ddotw(T, t, t);
      omega = ddotw(T, sv, t);
      if (tt != 0.0) omega /= tt;
      for (size_t k = 0; k < len; ++k) x[k] += omega * q[k];
      memcpy(b, sv, sizeof(double) * len);
      { const double a = -omega; for (size_t k = 0; k < len; ++k) b[k] += a * t[k]; }
      rho = rho_new;
      orc_nrm2x(T, b, last);
      ++nh;
      if (hist) for (int k = 0; k < s; ++k) hist[(size_t)nh * s + k] = last[k];
      ++iters;
      if (sc_cmp(last, abslimit, s) || sc_cmp(last, reach, s)) { *converged = 1; break; }
      if (sc_eq(last, old, 1e-4, s)) eq_count++;
      else eq_count = 0;
      for (int k = 0; k < s; ++k) old[k] = last[k];
      if (eq_count > 4) { *converged = 0; break; }
    }
  }
done:
  free(r); free(p); free(v); free(sv); free(t); free(q);
  ws_free(&w);
  free(scratch);
  return rc ? rc : iters;
}

/* SetSurfaceClasses, gm/algebra.cc:2838-2925: FINE_GRID_DOF = VCLASS >= 2 and
 * VNCLASS <= 1; FULLREFINELEVEL = the lowest level holding such a vector
 * (the top level if none does). */
static int fine_grid_dof(const orc_level *L, int i) { return L->vclass[i] >= NEWDEF_CLASS && L->vnclass[i] <= 1; }
int orc_fullrefinelevel(const orc_mg *mg) {
  const int top = mg->nlevels - 1;
  int frl = top;
  for (int l = top; l >= 0; --l)
    for (int i = 0; i < mg->lev[l].n; ++i)
      if (fine_grid_dof(&mg->lev[l], i)) { frl = l; break; }
  return frl;
}

/* ON_SURFACE row set (np/algebra/vecloop.ct, matloop.ct): FINE_GRID_DOF rows of
 * the levels FULLREFINELEVEL..top-1, then NEW_DEFECT rows of the top level */
static int surface_row(const orc_level *L, int i, int is_top) {
  return is_top ? L->vclass[i] >= NEWDEF_CLASS : fine_grid_dof(L, i);
}

/* dmatmul_minus ON_SURFACE, ugblas.cc:3997: b -= A x on the surface rows,
 * each with its own level's matrix and x */
static void surface_defect(const orc_mg *mg, int frl, double *const *b, double *const *x) {
  const int top = mg->nlevels - 1;
  for (int l = frl; l <= top; ++l) {
    const orc_level *L = &mg->lev[l];
    const int s = L->s;
    for (int i = 0; i < L->n; ++i) {
      if (!surface_row(L, i, l == top)) continue;
      for (int k = L->rowptr[i]; k < L->rowptr[i + 1]; ++k) {
        const double *m = L->val + (size_t)k * s * s, *yj = x[l] + (size_t)L->col[k] * s;
        for (int r = 0; r < s; ++r) {
          double acc = 0.0;
          for (int c = 0; c < s; ++c) acc += m[r * s + c] * yj[c];
          b[l][(size_t)i * s + r] -= acc;
        }
      }
    }
  }
}

/* dnrm2x ON_SURFACE, ugblas.cc:3156: sums of squares in the loop order above */
static void surface_norm(const orc_mg *mg, int frl, double *const *b, double *out) {
  const int top = mg->nlevels - 1;
  const int s = mg->lev[top].s;
  for (int r = 0; r < s; ++r) out[r] = 0.0;
  for (int l = frl; l <= top; ++l) {
    const orc_level *L = &mg->lev[l];
    for (int i = 0; i < L->n; ++i) {
      if (!surface_row(L, i, l == top)) continue;
      for (int r = 0; r < s; ++r) { double v = b[l][(size_t)i * s + r]; out[r] += v * v; }
    }
  }
  for (int r = 0; r < s; ++r) out[r] = sqrt(out[r]);
}

int orc_ls_solve_levels(const orc_mg *mg, double *const *x, double *const *b, const double *red,
                        const double *abslimit, int maxit, double *hist, int *converged) {
  const int top = mg->nlevels - 1;
  const int s = mg->lev[top].s;
  const int bl = mg->baselevel < top ? mg->baselevel : top;
  const int frl = orc_fullrefinelevel(mg);
  orc_ws w;
  int rc = ws_init_levels(&w, mg, b), it = 0;
  *converged = 0;
  if (rc) goto done;
  {
    double first[ORC_MAX_S], last[ORC_MAX_S], reach[ORC_MAX_S];
    surface_defect(mg, frl, b, x);
    surface_norm(mg, frl, b, first);
    if (hist) for (int r = 0; r < s; ++r) hist[r] = first[r];
    for (int r = 0; r < s; ++r) { reach[r] = first[r] * red[r]; if (reach[r] == 0.0) reach[r] = red[r]; }
    *converged = sc_cmp(first, abslimit, s);
    for (it = 0; it < maxit; ++it) {
      if (*converged) break;
      memset(w.c[top], 0, sizeof(double) * (size_t)mg->lev[top].n * s);
      if ((rc = lmgc(&w, top))) goto done;
      for (int l = bl; l <= top; ++l) vadd(x[l], w.c[l], (size_t)mg->lev[l].n * s); /* LSUpdate, ls.cc:869 */
      surface_norm(mg, frl, b, last);
      if (hist) for (int r = 0; r < s; ++r) hist[(size_t)(it + 1) * s + r] = last[r];
      if (sc_cmp(last, abslimit, s) || sc_cmp(last, reach, s)) { *converged = 1; ++it; break; }
    }
  }
done:
  ws_free(&w);
  return rc ? rc : it;
}

/* ---- Krylov solvers over the levels baselevel..top of a locally refined
 * hierarchy: vector operations ALL_VECTORS on every level, products ON_SURFACE */

/* ddot / ddotw ON_SURFACE (ugblas.cc:3104 / 3023): the surface rows in the
 * loop order of matloop.ct; ddot sums every component into one sum, ddotw
 * (weights 1) per component, then adds the components */
static double surface_ddot(const orc_mg *mg, int frl, double *const *x, double *const *y, int weighted) {
  const int top = mg->nlevels - 1, s = mg->lev[top].s;
  double sum = 0.0, a[ORC_MAX_S] = {0};
  for (int l = frl; l <= top; ++l) {
    const orc_level *L = &mg->lev[l];
    for (int i = 0; i < L->n; ++i) {
      if (!surface_row(L, i, l == top)) continue;
      for (int r = 0; r < s; ++r) {
        const double v = x[l][(size_t)i * s + r] * y[l][(size_t)i * s + r];
        if (weighted) a[r] += v; else sum += v;
      }
    }
  }
  if (weighted)
    for (int r = 0; r < s; ++r) sum += 1.0 * a[r];
  return sum;
}

/* dmatmul ON_SURFACE (x = A y on the surface rows only, the other rows keep
 * their values) or ALL_VECTORS on the levels bl..top */
static void levels_matmul(const orc_mg *mg, int frl, int bl, int surface, double *const *x, double *const *y) {
  const int top = mg->nlevels - 1;
  for (int l = surface ? frl : bl; l <= top; ++l) {
    const orc_level *L = &mg->lev[l];
    const int s = L->s, ss = s * s;
    for (int i = 0; i < L->n; ++i) {
      if (surface && !surface_row(L, i, l == top)) continue;
      double acc[ORC_MAX_S] = {0};
      for (int k = L->rowptr[i]; k < L->rowptr[i + 1]; ++k) {
        const double *m = L->val + (size_t)k * ss, *w = y[l] + (size_t)L->col[k] * s;
        for (int r = 0; r < s; ++r) {
          double t = 0.0;
          for (int c = 0; c < s; ++c) t += m[r * s + c] * w[c];
          acc[r] += t;
        }
      }
      for (int r = 0; r < s; ++r) x[l][(size_t)i * s + r] = acc[r];
    }
  }
}

typedef struct {
  int nl;
  double *v[32];
} orc_lvec; /* one vector on every level (NULL below bl) */

static int lvec_alloc(const orc_mg *mg, int bl, orc_lvec *v) {
  memset(v, 0, sizeof *v);
  v->nl = mg->nlevels;
  if (mg->nlevels > 32) return -1;
  for (int l = bl; l < mg->nlevels; ++l)
    if (!(v->v[l] = (double *)calloc((size_t)mg->lev[l].n * mg->lev[l].s, sizeof(double)))) return -1;
  return 0;
}
static void lvec_free(orc_lvec *v) { for (int l = 0; l < v->nl; ++l) free(v->v[l]); }
static size_t lvlen(const orc_mg *mg, int l) { return (size_t)mg->lev[l].n * mg->lev[l].s; }

/* the lmgc preconditioner on a copy of d (every level): q = c */
static int precond_levels(orc_ws *w, int bl, double *const *q, double *const *d) {
  const orc_mg *mg = w->mg;
  const int top = mg->nlevels - 1;
  for (int l = bl; l <= top; ++l) memcpy(w->b[l], d[l], sizeof(double) * lvlen(mg, l));
  memset(w->c[top], 0, sizeof(double) * lvlen(mg, top));
  int rc = lmgc(w, top);
  for (int l = bl; l <= top; ++l) memcpy(q[l], w->c[l], sizeof(double) * lvlen(mg, l));
  return rc;
}

int orc_cg_solve_levels(const orc_mg *mg, double *const *x, double *const *b, const double *red,
                        const double *abslimit, int maxit, double *hist, int *converged) {
  const int top = mg->nlevels - 1, s = mg->lev[top].s;
  const int bl = mg->baselevel < top ? mg->baselevel : top;
  const int frl = orc_fullrefinelevel(mg);
  orc_ws w;
  orc_lvec p, t;
  if (frl < bl) return -3000000; /* the surface would reach below the allocated levels */
  int rc = ws_init_levels(&w, mg, b), it = 0;
  if (!rc) rc = lvec_alloc(mg, bl, &p);
  if (!rc) rc = lvec_alloc(mg, bl, &t);
  *converged = 0;
  if (rc) goto done;
  {
    double first[ORC_MAX_S], last[ORC_MAX_S], reach[ORC_MAX_S], rho = 1.0; /* CGPrepare, ls.cc:976 */
    surface_defect(mg, frl, b, x);
    surface_norm(mg, frl, b, first);
    if (hist) for (int r = 0; r < s; ++r) hist[r] = first[r];
    for (int r = 0; r < s; ++r) { reach[r] = first[r] * red[r]; if (reach[r] == 0.0) reach[r] = red[r]; }
    *converged = sc_cmp(first, abslimit, s);
    for (it = 0; it < maxit; ++it) {
      if (*converged) break;
      memset(w.c[top], 0, sizeof(double) * lvlen(mg, top));
      if ((rc = lmgc(&w, top))) goto done;
      /* CGUpdate, ls.cc:989-1030 on the levels bl..top */
      double *const *c = w.c;
      levels_matmul(mg, frl, bl, 0, t.v, c);
      for (int l = bl; l <= top; ++l) vadd(b[l], t.v[l], lvlen(mg, l));
      double lambda = surface_ddot(mg, frl, c, b, 0);
      const double f = lambda / rho;
      for (int l = bl; l <= top; ++l) for (size_t i = 0; i < lvlen(mg, l); ++i) p.v[l][i] *= f;
      rho = lambda;
      for (int l = bl; l <= top; ++l) vadd(p.v[l], c[l], lvlen(mg, l));
      levels_matmul(mg, frl, bl, 0, t.v, p.v);
      lambda = surface_ddot(mg, frl, t.v, p.v, 0);
      if (lambda == 0.0) { rc = -2000000; goto done; }
      const double a = rho / lambda, na = -rho / lambda;
      for (int l = bl; l <= top; ++l)
        for (size_t i = 0; i < lvlen(mg, l); ++i) { x[l][i] += a * p.v[l][i]; }
      for (int l = bl; l <= top; ++l)
        for (size_t i = 0; i < lvlen(mg, l); ++i) { b[l][i] += na * t.v[l][i]; }
      surface_norm(mg, frl, b, last);
      if (hist) for (int r = 0; r < s; ++r) hist[(size_t)(it + 1) * s + r] = last[r];
      if (sc_cmp(last, abslimit, s) || sc_cmp(last, reach, s)) { *converged = 1; ++it; break; }
    }
  }
done:
  lvec_free(&p); lvec_free(&t);
  ws_free(&w);
  return rc ? rc : it;
}

int orc_bcgs_solve_levels(const orc_mg *mg, double *const *x, double *const *b, const double *red,
                          const double *abslimit, int maxit, double *hist, int *converged) {
  const int top = mg->nlevels - 1, s = mg->lev[top].s;
  const int bl = mg->baselevel < top ? mg->baselevel : top;
  const int frl = orc_fullrefinelevel(mg);
  orc_ws w;
  orc_lvec r, p, v, sv, t, q;
  double *scratch[32] = {0};
  int rc = 0, iters = 0;
  *converged = 0;
  if (mg->nlevels > 32) return -1;
  if (frl < bl) return -3000000;
  for (int l = bl; l <= top; ++l) scratch[l] = (double *)calloc(lvlen(mg, l), sizeof(double));
  rc = ws_init_levels(&w, mg, scratch);
  if (!rc) rc = lvec_alloc(mg, bl, &r);
  if (!rc) rc = lvec_alloc(mg, bl, &p);
  if (!rc) rc = lvec_alloc(mg, bl, &v);
  if (!rc) rc = lvec_alloc(mg, bl, &sv);
  if (!rc) rc = lvec_alloc(mg, bl, &t);
  if (!rc) rc = lvec_alloc(mg, bl, &q);
  if (rc) goto done;
  {
    double first[ORC_MAX_S], last[ORC_MAX_S], reach[ORC_MAX_S], old[ORC_MAX_S];
    double alpha = 0.0, rho_new = 0.0, beta = 0.0, tt = 0.0, rho = 0.0, omega = 0.0;
    int restart = 1, eq_count = 0, nh = 0;
    for (int k = 0; k < s; ++k) old[k] = -1.0; /* BCGSPreProcess, ls.cc:1831 */
    surface_defect(mg, frl, b, x);
    surface_norm(mg, frl, b, first);
    if (hist) for (int k = 0; k < s; ++k) hist[k] = first[k];
    for (int k = 0; k < s; ++k) { reach[k] = first[k] * red[k]; if (reach[k] == 0.0) reach[k] = red[k]; }
    *converged = sc_cmp(first, abslimit, s);
    /* BCGSSolver, ls.cc:1864-2062 on the levels bl..top (no restart index, weights 1) */
    for (int i = 0; i < maxit; ++i) {
      if (*converged) break;
      if (restart) {
        for (int l = bl; l <= top; ++l) {
          memset(p.v[l], 0, sizeof(double) * lvlen(mg, l));
          memset(v.v[l], 0, sizeof(double) * lvlen(mg, l));
          memcpy(r.v[l], b[l], sizeof(double) * lvlen(mg, l));
        }
        alpha = rho = omega = 1.0;
        restart = 0;
      }
      rho_new = surface_ddot(mg, frl, b, r.v, 1);
      if (rho != 0.0 && omega != 0.0) beta = rho_new * alpha / rho / omega;
      for (int l = bl; l <= top; ++l) {
        const size_t n = lvlen(mg, l);
        for (size_t k = 0; k < n; ++k) p.v[l][k] *= beta;
        vadd(p.v[l], b[l], n);
        const double a = -beta * omega;
        for (size_t k = 0; k < n; ++k) p.v[l][k] += a * v.v[l][k];
      }
      if ((rc = precond_levels(&w, bl, q.v, p.v))) goto done;
      levels_matmul(mg, frl, bl, 1, v.v, q.v);
      alpha = surface_ddot(mg, frl, v.v, r.v, 1);
      if (alpha != 0.0) alpha = rho_new / alpha;
      for (int l = bl; l <= top; ++l)
        for (size_t k = 0; k < lvlen(mg, l); ++k) x[l][k] += alpha * q.v[l][k];
      ++iters;
      for (int l = bl; l <= top; ++l) {
        const size_t n = lvlen(mg, l);
        memcpy(sv.v[l], b[l], sizeof(double) * n);
        const double a = -alpha;
        for (size_t k = 0; k < n; ++k) sv.v[l][k] += a * v.v[l][k];
      }
      surface_norm(mg, frl, sv.v, last);
      ++nh;
      if (hist) for (int k = 0; k < s; ++k) hist[(size_t)nh * s + k] = last[k];
      if (sc_cmp(last, abslimit, s) || sc_cmp(last, reach, s)) {
        for (int l = bl; l <= top; ++l) memcpy(b[l], sv.v[l], sizeof(double) * lvlen(mg, l));
        *converged = 1;
        break;
      }
      if ((rc = precond_levels(&w, bl, q.v, sv.v))) goto done;
      levels_matmul(mg, frl, bl, 1, t.v, q.v);
      tt = surface_ddot(mg, frl, t.v, t.v, 1);
      omega = surface_ddot(mg, frl, sv.v, t.v, 1);
      if (tt != 0.0) omega /= tt;
      for (int l = bl; l <= top; ++l) {
        const size_t n = lvlen(mg, l);
        for (size_t k = 0; k < n; ++k) x[l][k] += omega * q.v[l][k];
        memcpy(b[l], sv.v[l], sizeof(double) * n);
        const double a = -omega;
        for (size_t k = 0; k < n; ++k) b[l][k] += a * t.v[l][k];
      }
      rho = rho_new;
      surface_norm(mg, frl, b, last);
      ++nh;
      if (hist) for (int k = 0; k < s; ++k) hist[(size_t)nh * s + k] = last[k];
      ++iters;
      if (sc_cmp(last, abslimit, s) || sc_cmp(last, reach, s)) { *converged = 1; break; }
      if (sc_eq(last, old, 1e-4, s)) eq_count++;
      else eq_count = 0;
      for (int k = 0; k < s; ++k) old[k] = last[k];
      if (eq_count > 4) { *converged = 0; break; }
    }
  }
done:
  lvec_free(&r); lvec_free(&p); lvec_free(&v); lvec_free(&sv); lvec_free(&t); lvec_free(&q);
  ws_free(&w);
  for (int l = 0; l < 32; ++l) free(scratch[l]);
  return rc ? rc : iters;
}

int orc_ls_solve(const orc_mg *mg, double *x, double *b, const double *red, const double *abslimit, int maxit,
                 double *hist, int *converged) {
  const int top = mg->nlevels - 1;
  const int s = mg->lev[top].s;
  orc_ws w;
  int rc = ws_init(&w, mg, b), it = 0;
  *converged = 0;
  if (rc) goto done;
  {
    const orc_level *T = &mg->lev[top];
    const size_t len = (size_t)T->n * s;
    double first[ORC_MAX_S], last[ORC_MAX_S], reach[ORC_MAX_S];
    orc_matmul_minus(T, b, x);
    orc_nrm2x(T, b, first);
    if (hist) for (int r = 0; r < s; ++r) hist[r] = first[r];
    for (int r = 0; r < s; ++r) { reach[r] = first[r] * red[r]; if (reach[r] == 0.0) reach[r] = red[r]; }
    *converged = sc_cmp(first, abslimit, s);
    for (it = 0; it < maxit; ++it) {
      if (*converged) break;
      memset(w.c[top], 0, sizeof(double) * len);
      if ((rc = lmgc(&w, top))) goto done;
      vadd(x, w.c[top], len); /* coarse-level x copies are not materialised */
      orc_nrm2x(T, b, last);
      if (hist) for (int r = 0; r < s; ++r) hist[(size_t)(it + 1) * s + r] = last[r];
      if (sc_cmp(last, abslimit, s) || sc_cmp(last, reach, s)) { *converged = 1; ++it; break; }
    }
  }
done:
  ws_free(&w);
  return rc ? rc : it;
}
