// Eigenpairs of the small symmetric subspace matrix of the Davidson solver: the eigen-solve
// of PsociGAsubspace::diagSubspaceGOP (PsociGAsubspace.C:1088-1171), which calls LAPACK
// dsygv with the overlap matrix as metric.  The device basis is orthonormal, so the metric
// is the identity and the problem is the standard symmetric one.
//
// Method (Golub & Van Loan, "Matrix Computations", sections 8.3.1-8.3.3): Householder
// reduction to tridiagonal form with the orthogonal factor accumulated, then implicit
// symmetric QR steps with the Wilkinson shift (Givens bulge chasing) on the tridiagonal,
// the rotations applied to the factor; eigenpairs sorted by ascending eigenvalue.  For the
// orders the solver uses (at most 96) this is a fraction of a millisecond of host time,
// against the FP64 pipe of one SM for a device Jacobi.
//
// Host code only: no device, no stream.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

#include "../../include/psoci_gpu.h"

extern "C" psoci_status psoci_subspace_eigen(int n, const double *G, int ldg, double *w, double *Y, int ldy) {
  if (n < 1 || !G || !w || !Y || ldg < n || ldy < n) return PSOCI_ERR_INVALID_ARG;
  // a: symmetric copy (the halves averaged), row-major n x n; q: accumulated factor, stored
  // by columns (q[k*n + r] = Q(r, k)) so that a rotation or reflection streams whole columns
  std::vector<double> a((size_t)n * n), q((size_t)n * n, 0.0), d(n), e(n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const double x = G[(size_t)i * ldg + j], y = G[(size_t)j * ldg + i];
      if (!std::isfinite(x)) return PSOCI_ERR_NUMERIC;
      a[(size_t)i * n + j] = 0.5 * (x + y);
    }
  for (int i = 0; i < n; ++i) q[(size_t)i * n + i] = 1.0;
  auto A = [&](int i, int j) -> double & { return a[(size_t)i * n + j]; };
  auto Qc = [&](int k) -> double * { return q.data() + (size_t)k * n; };  // column k of Q

  // 1. tridiagonalise: P_k = I - beta v v^T zeroes column k below the subdiagonal
  std::vector<double> v(n), p(n), wv(n);
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;  // order of the trailing block, rows k+1..n-1
    double xn = 0.0;
    for (int i = 0; i < m; ++i) xn += A(k + 1 + i, k) * A(k + 1 + i, k);
    xn = std::sqrt(xn);
    if (xn == 0.0) continue;
    const double x0 = A(k + 1, k);
    const double alpha = (x0 > 0.0) ? -xn : xn;  // v0 = x0 - alpha without cancellation
    for (int i = 0; i < m; ++i) v[i] = A(k + 1 + i, k);
    v[0] -= alpha;
    double vv = 0.0;
    for (int i = 0; i < m; ++i) vv += v[i] * v[i];
    if (vv == 0.0) continue;
    const double beta = 2.0 / vv;
    // trailing block B <- P B P = B - v w^T - w v^T, p = beta B v, w = p - (beta/2)(p.v) v
    double pv = 0.0;
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int j = 0; j < m; ++j) s += A(k + 1 + i, k + 1 + j) * v[j];
      p[i] = beta * s;
      pv += p[i] * v[i];
    }
    const double kf = 0.5 * beta * pv;
    for (int i = 0; i < m; ++i) wv[i] = p[i] - kf * v[i];
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) A(k + 1 + i, k + 1 + j) -= v[i] * wv[j] + wv[i] * v[j];
    A(k + 1, k) = A(k, k + 1) = alpha;
    for (int i = 1; i < m; ++i) A(k + 1 + i, k) = A(k, k + 1 + i) = 0.0;
    // Q <- Q P on columns k+1..n-1: u = beta Q v, then column j -= v_j u
    std::fill(p.begin(), p.end(), 0.0);
    for (int j = 0; j < m; ++j) {
      const double *qj = Qc(k + 1 + j);
      const double vj = v[j];
      for (int r = 0; r < n; ++r) p[r] += qj[r] * vj;
    }
    for (int j = 0; j < m; ++j) {
      double *qj = Qc(k + 1 + j);
      const double f = beta * v[j];
      for (int r = 0; r < n; ++r) qj[r] -= f * p[r];
    }
  }
  for (int i = 0; i < n; ++i) d[i] = A(i, i);
  for (int i = 0; i + 1 < n; ++i) e[i] = A(i + 1, i);

  // 2. implicit symmetric QR with the Wilkinson shift; e[i] couples d[i] and d[i+1]
  auto small = [&](int i) {
    return std::fabs(e[i]) <= DBL_EPSILON * (std::fabs(d[i]) + std::fabs(d[i + 1])) || std::fabs(e[i]) < DBL_MIN;
  };
  int hi = n - 1, steps = 0;
  while (hi > 0) {
    if (small(hi - 1)) {
      e[hi - 1] = 0.0;
      --hi;
      continue;
    }
    if (++steps > 60 * n) return PSOCI_ERR_NUMERIC;
    int lo = hi - 1;
    while (lo > 0 && !small(lo - 1)) --lo;
    // shift: the eigenvalue of the trailing 2 x 2 block closer to d[hi]
    const double dd = 0.5 * (d[hi - 1] - d[hi]), eh = e[hi - 1];
    const double den = dd + (dd >= 0.0 ? 1.0 : -1.0) * std::sqrt(dd * dd + eh * eh);
    const double mu = d[hi] - eh * (eh / den);
    double x = d[lo] - mu, z = e[lo];
    for (int k = lo; k < hi; ++k) {
      // rotation G = [c -s; s c] on (k, k+1) with G^T (x, z) = (r, 0)
      const double r = std::sqrt(x * x + z * z);  // subspace matrices are far from overflow
      const double c = (r == 0.0) ? 1.0 : x / r, s = (r == 0.0) ? 0.0 : z / r;
      if (k > lo) e[k - 1] = r;  // the bulge at (k+1, k-1) folded into e[k-1]
      const double a0 = d[k], b0 = e[k], c0 = d[k + 1];
      d[k] = c * c * a0 + 2.0 * c * s * b0 + s * s * c0;
      d[k + 1] = s * s * a0 - 2.0 * c * s * b0 + c * c * c0;
      e[k] = c * s * (c0 - a0) + (c * c - s * s) * b0;
      if (k + 1 < hi) {
        const double f = e[k + 1];
        z = s * f;  // new bulge at (k+2, k)
        e[k + 1] = c * f;
        x = e[k];
      }
      double *q0 = Qc(k), *q1 = Qc(k + 1);
      for (int rr = 0; rr < n; ++rr) {
        const double qk = q0[rr], qk1 = q1[rr];
        q0[rr] = c * qk + s * qk1;
        q1[rr] = -s * qk + c * qk1;
      }
    }
  }

  // 3. ascending order (ties keep the index order)
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
  for (int c = 0; c < n; ++c) {
    w[c] = d[idx[c]];
    const double *qc = Qc(idx[c]);
    for (int r = 0; r < n; ++r) Y[(size_t)r * ldy + c] = qc[r];
  }
  return PSOCI_OK;
}
