// Host eigensolver of the Davidson subspace matrix: the k lowest eigenpairs
// of a symmetric m x m matrix (m <= a few hundred).
//
// Householder reduction to tridiagonal form, Sturm-sequence bisection for the
// k smallest eigenvalues, inverse iteration on the tridiagonal matrix for
// their vectors (re-orthogonalised within clusters of close eigenvalues), and
// back-transformation by the Householder reflectors -- the classical
// Givens/Householder/Wilkinson scheme.  Only the k wanted pairs are computed,
// which is what the Davidson iteration reads (Ritz values, Ritz vector
// coefficients and the locking weights of the lowest nroots roots,
// src/Davidson.cpp:224-260): O(4/3 m^3) for the reduction, O(k m) for the
// tridiagonal work and O(k m^2) for the back-transformation.
#include <algorithm>
#include <cmath>
#include <vector>

namespace pg {

namespace {

// Band storage of the pivoted LU factor of T - lambda I, kept across calls.
struct TridiagScratch {
  std::vector<double> u0, u1, u2, l;
  std::vector<char> swapped;
  explicit TridiagScratch(int m) : u0(m), u1(m), u2(m), l(m), swapped(m) {}
};

// Factor T - lambda I (tridiagonal T) by Gaussian elimination with partial
// pivoting into ts; a tiny pivot is replaced by eps*|T|.
void tridiag_factor(int m, const double* d, const double* e, double lambda, double tiny, TridiagScratch& ts) {
  // bands of the factor: u0 (diagonal), u1, u2 (two super-diagonals after pivoting)
  double *u0 = ts.u0.data(), *u1 = ts.u1.data(), *u2 = ts.u2.data(), *l = ts.l.data();
  char* swapped = ts.swapped.data();
  std::fill(swapped, swapped + m, 0);
  double diag = d[0] - lambda;
  double sup = m > 1 ? e[0] : 0.0;
  for (int i = 0; i < m - 1; ++i) {
    const double sub = e[i];
    const double nd = d[i + 1] - lambda;
    const double ns = i + 1 < m - 1 ? e[i + 1] : 0.0;
    if (fabs(diag) >= fabs(sub)) {  // no swap
      double piv = diag != 0 ? diag : tiny;
      const double f = sub / piv;
      u0[i] = piv;
      u1[i] = sup;
      u2[i] = 0.0;
      l[i] = f;
      diag = nd - f * sup;
      sup = ns;
    } else {  // swap rows i, i+1
      const double f = diag / sub;
      u0[i] = sub;
      u1[i] = nd;
      u2[i] = ns;
      l[i] = f;
      swapped[i] = 1;
      diag = sup - f * nd;
      sup = -f * ns;
    }
  }
  u0[m - 1] = diag != 0 ? diag : tiny;
}

// Solve (T - lambda I) y = b in place with the factor of tridiag_factor.
void tridiag_solve(int m, double tiny, double* b, const TridiagScratch& ts) {
  const double *u0 = ts.u0.data(), *u1 = ts.u1.data(), *u2 = ts.u2.data(), *l = ts.l.data();
  const char* swapped = ts.swapped.data();
  // forward: apply L^-1 with the row swaps
  for (int i = 0; i < m - 1; ++i) {
    if (swapped[i]) std::swap(b[i], b[i + 1]);
    b[i + 1] -= l[i] * b[i];
  }
  // back substitution with U
  for (int i = m - 1; i >= 0; --i) {
    double s = b[i];
    if (i + 1 < m) s -= u1[i] * b[i + 1];
    if (i + 2 < m) s -= u2[i] * b[i + 2];
    const double p = u0[i] != 0 ? u0[i] : tiny;
    b[i] = s / p;
  }
}

}  // namespace

// k lowest eigenpairs of the symmetric matrix given by the upper triangle of
// S (column-major, leading dimension ld).  Eigenvalues ascending into w[k];
// eigenvectors into V (column j at V + j*ldv).  False on non-finite input.
bool lowest_eigenpairs(int m, const double* S, int ld, int k, double* w, double* V, int ldv) {
  if (k > m) k = m;
  std::vector<double> a((size_t)m * m);  // full symmetric copy, row-major (same as col-major)
  for (int j = 0; j < m; ++j)
    for (int i = 0; i <= j; ++i) {
      const double v = S[i + (size_t)j * ld];
      if (!std::isfinite(v)) return false;
      a[(size_t)i * m + j] = a[(size_t)j * m + i] = v;
    }
  if (m == 1) {
    w[0] = a[0];
    V[0] = 1.0;
    return true;
  }
  // --- Householder tridiagonalisation: for each column c, a reflector
  // H = I - beta v v^T zeroes a[c+2.., c]; reflectors are kept in hv/hb.
  std::vector<double> hv((size_t)m * m, 0.0), hb(m, 0.0), p(m), q(m);
  std::vector<double> d(m), e(m, 0.0);
  for (int c = 0; c < m - 2; ++c) {
    const int n1 = m - c - 1;  // length of the column below the diagonal
    double* v = hv.data() + (size_t)c * m + (c + 1);
    double alpha2 = 0;
    for (int i = 0; i < n1; ++i) {
      v[i] = a[(size_t)(c + 1 + i) * m + c];
      alpha2 += v[i] * v[i];
    }
    const double x0 = v[0];
    double tail = alpha2 - x0 * x0;
    if (tail <= 1e-300 * alpha2 || tail == 0) {  // already tridiagonal in this column
      hb[c] = 0;
      e[c] = x0;
      continue;
    }
    const double alpha = x0 >= 0 ? -sqrt(alpha2) : sqrt(alpha2);
    v[0] = x0 - alpha;
    const double vtv = v[0] * v[0] + tail;
    const double beta = 2.0 / vtv;
    hb[c] = beta;
    e[c] = alpha;
    // trailing block A22 <- H A22 H = A22 - v w^T - w v^T,
    // p = beta A22 v, w = p - (beta/2)(p^T v) v
    double* A22 = a.data() + (size_t)(c + 1) * m + (c + 1);
    // p = A22 v as a sum of rows: A22 is exactly symmetric (the rank-2 update
    // below adds the same two products for (i, j) and (j, i)), so p_i is the
    // same sum, in the same order of j, as the row-times-vector dot product,
    // while the inner loop runs over independent i (it vectorises)
    for (int i = 0; i < n1; ++i) p[i] = 0.0;
    for (int j = 0; j < n1; ++j) {
      const double vj = v[j];
      const double* row = A22 + (size_t)j * m;
      for (int i = 0; i < n1; ++i) p[i] += row[i] * vj;
    }
    for (int i = 0; i < n1; ++i) p[i] *= beta;
    double pv = 0;
    for (int i = 0; i < n1; ++i) pv += p[i] * v[i];
    const double half = 0.5 * beta * pv;
    for (int i = 0; i < n1; ++i) q[i] = p[i] - half * v[i];
    for (int i = 0; i < n1; ++i) {
      double* row = A22 + (size_t)i * m;
      const double vi = v[i], qi = q[i];
      for (int j = 0; j < n1; ++j) row[j] -= vi * q[j] + qi * v[j];
    }
  }
  for (int i = 0; i < m; ++i) d[i] = a[(size_t)i * m + i];
  e[m - 2] = a[(size_t)(m - 1) * m + (m - 2)];
  // e[c] is T(c+1, c) for c < m-1
  std::vector<double> e2(m, 0.0);
  double tnorm = 0;
  for (int i = 0; i < m; ++i) {
    const double ei = i < m - 1 ? fabs(e[i]) : 0.0;
    const double em = i > 0 ? fabs(e[i - 1]) : 0.0;
    tnorm = std::max(tnorm, fabs(d[i]) + ei + em);
    if (i < m - 1) e2[i] = e[i] * e[i];
  }
  if (!std::isfinite(tnorm)) return false;
  if (tnorm == 0) tnorm = 1;
  // --- bisection for the k smallest eigenvalues (Gershgorin bracket)
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < m; ++i) {
    const double r = (i < m - 1 ? fabs(e[i]) : 0.0) + (i > 0 ? fabs(e[i - 1]) : 0.0);
    lo = std::min(lo, d[i] - r);
    hi = std::max(hi, d[i] + r);
  }
  const double eps = 2.2e-16;
  lo -= 4 * eps * tnorm;
  hi += 4 * eps * tnorm;
  const double tol = eps * tnorm;
  // All k brackets at once: each round evaluates the Sturm counts at the
  // midpoints of the brackets still open in one pass over the tridiagonal
  // (their division chains are independent and overlap), and each count c at
  // x narrows every bracket: eigenvalues 0 .. c-1 lie below x, the rest not.
  {
    std::vector<double> blo(k, lo), bhi(k, hi), mids(k), qv(k);
    std::vector<int> cnt(k);
    for (int round = 0; round < 200; ++round) {
      int no = 0;
      for (int j = 0; j < k; ++j) {
        const double mid = 0.5 * (blo[j] + bhi[j]);
        if (bhi[j] - blo[j] > tol && mid != blo[j] && mid != bhi[j]) mids[no++] = mid;
      }
      if (no == 0) break;
      for (int t = 0; t < no; ++t) {
        qv[t] = d[0] - mids[t];
        cnt[t] = qv[t] < 0 ? 1 : 0;
      }
      for (int i = 1; i < m; ++i) {
        const double di = d[i], ei2 = e2[i - 1];
        for (int t = 0; t < no; ++t) {
          const double prev = qv[t] != 0 ? qv[t] : 1e-300;
          qv[t] = di - mids[t] - ei2 / prev;
          cnt[t] += qv[t] < 0 ? 1 : 0;
        }
      }
      for (int t = 0; t < no; ++t)
        for (int j = 0; j < k; ++j) {
          if (j < cnt[t]) bhi[j] = std::min(bhi[j], mids[t]);
          else blo[j] = std::max(blo[j], mids[t]);
        }
    }
    for (int j = 0; j < k; ++j) w[j] = 0.5 * (blo[j] + bhi[j]);
  }
  // --- inverse iteration on the tridiagonal for each wanted vector
  std::vector<double> y((size_t)k * m);
  const double tiny = eps * tnorm;
  TridiagScratch ts(m);
  for (int j = 0; j < k; ++j) {
    double* yj = y.data() + (size_t)j * m;
    // deterministic, non-degenerate start
    for (int i = 0; i < m; ++i) yj[i] = 1.0 + 0.1 * std::sin(1.0 + 0.7 * i + 1.3 * j);
    const double shift = w[j];
    tridiag_factor(m, d.data(), e.data(), shift, tiny, ts);  // one factor for the four solves
    for (int it = 0; it < 4; ++it) {
      tridiag_solve(m, tiny, yj, ts);
      // orthogonalise against the earlier vectors (needed inside clusters of
      // close eigenvalues, harmless elsewhere)
      for (int r = 0; r < j; ++r) {
        const double* yr = y.data() + (size_t)r * m;
        double s = 0;
        for (int i = 0; i < m; ++i) s += yr[i] * yj[i];
        for (int i = 0; i < m; ++i) yj[i] -= s * yr[i];
      }
      double nrm = 0;
      for (int i = 0; i < m; ++i) nrm += yj[i] * yj[i];
      nrm = sqrt(nrm);
      if (!(nrm > 0) || !std::isfinite(nrm)) return false;
      for (int i = 0; i < m; ++i) yj[i] /= nrm;
    }
  }
  // --- back-transformation: x = H_0 H_1 ... H_{m-3} y
  for (int j = 0; j < k; ++j) {
    double* x = y.data() + (size_t)j * m;
    for (int c = m - 3; c >= 0; --c) {
      if (hb[c] == 0) continue;
      const double* v = hv.data() + (size_t)c * m + (c + 1);
      const int n1 = m - c - 1;
      double s = 0;
      for (int i = 0; i < n1; ++i) s += v[i] * x[c + 1 + i];
      s *= hb[c];
      for (int i = 0; i < n1; ++i) x[c + 1 + i] -= s * v[i];
    }
    for (int i = 0; i < m; ++i) V[i + (size_t)j * ldv] = x[i];
  }
  return true;
}

}  // namespace pg

#include "pisces_gb300.h"

extern "C" pg_status pg_subspace_lowest(int m, const double* S, int ld, int k, double* w, double* V, int ldv) {
  if (m <= 0 || k <= 0 || k > m || ld < m || ldv < m || !S || !w || !V) return PG_BAD_ARG;
  return pg::lowest_eigenpairs(m, S, ld, k, w, V, ldv) ? PG_OK : PG_NUMERIC;
}
