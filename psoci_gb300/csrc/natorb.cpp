// Natural orbitals and occupations from a packed 1-particle density: the MO-basis part of
// PsociNOpopulations::constructNaturalOrbitals (PsociNOpopulations.C:569-669).
//
//   per symmetry block: unpack the square block from the packed triangle
//   (diagonalizeNOinMObasis, :456-467, twoDindex), solve D y = n y with a unit metric
//   (:469-494, dsygv ITYPE 1), order the pairs by occupation, largest first, keeping the
//   solver's order among equal occupations (sortNOinMObasis, :269-344, std::list::sort
//   with compare_evalues, :338-344).
//
// A block holds the orbitals that carry one symmetry label, in ascending orbital order; the
// blocks follow in ascending label order.  With MOs ordered by symmetry, as the reference's
// MO files are, this is its nstart/nsize split (:603-610).  The eigen-solver is the cyclic
// Jacobi method (Rutishauser's formulation, as in Golub & Van Loan, "Matrix Computations",
// section 8.5): the blocks are at most 128 x 128 and Jacobi gives small eigenvalues to
// high relative accuracy, which is what the small occupations need.
//
// Host code only: no device, no stream; runs where the library loads.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/psoci_gpu.h"

namespace {

// symmetric A (n x n row-major, overwritten) -> eigenvalues w, eigenvectors as columns of V
void jacobi_eigen(int n, std::vector<double> &A, std::vector<double> &w, std::vector<double> &V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  auto a = [&](int i, int j) -> double & { return A[(size_t)i * n + j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < n; ++i) {
      diag += a(i, i) * a(i, i);
      for (int j = i + 1; j < n; ++j) off += a(i, j) * a(i, j);
    }
    if (off == 0.0 || off <= 1e-34 * diag) break;
    for (int p = 0; p < n - 1; ++p) {
      for (int q = p + 1; q < n; ++q) {
        const double apq = a(p, q);
        if (apq == 0.0) continue;
        // skip rotations below the rounding of both diagonal entries (after a few sweeps)
        if (sweep > 3 && std::fabs(apq) * 1e18 <= std::fabs(a(p, p)) && std::fabs(apq) * 1e18 <= std::fabs(a(q, q))) {
          a(p, q) = a(q, p) = 0.0;
          continue;
        }
        const double theta = (a(q, q) - a(p, p)) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c, tau = s / (1.0 + c);
        const double app = a(p, p), aqq = a(q, q);
        a(p, p) = app - t * apq;
        a(q, q) = aqq + t * apq;
        a(p, q) = a(q, p) = 0.0;
        for (int r = 0; r < n; ++r) {
          if (r == p || r == q) continue;
          const double arp = a(r, p), arq = a(r, q);
          const double np_ = arp - s * (arq + tau * arp);
          const double nq_ = arq + s * (arp - tau * arq);
          a(r, p) = a(p, r) = np_;
          a(r, q) = a(q, r) = nq_;
        }
        for (int r = 0; r < n; ++r) {
          double &vp = V[(size_t)r * n + p], &vq = V[(size_t)r * n + q];
          const double x = vp, y = vq;
          vp = x - s * (y + tau * x);
          vq = y + s * (x - tau * y);
        }
      }
    }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = a(i, i);
}

}  // namespace

extern "C" psoci_status psoci_natural_orbitals(int nbf, const double *dens, const int32_t *orb_sym, double *occ,
                                               double *vecs, int32_t *orb_order) {
  if (nbf < 1 || !dens || !orb_sym || !occ || !vecs) return PSOCI_ERR_INVALID_ARG;
  std::vector<int> order(nbf);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return orb_sym[x] < orb_sym[y]; });
  if (orb_order) for (int i = 0; i < nbf; ++i) orb_order[i] = order[i];
  size_t eoff = 0, voff = 0;
  for (int b0 = 0; b0 < nbf;) {
    int b1 = b0;
    while (b1 < nbf && orb_sym[order[b1]] == orb_sym[order[b0]]) ++b1;
    const int n = b1 - b0;
    std::vector<double> A((size_t)n * n), w, V;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const int64_t p = order[b0 + i], q = order[b0 + j];
        const int64_t hi = p > q ? p : q, lo = p > q ? q : p;
        A[(size_t)i * n + j] = dens[hi * (hi + 1) / 2 + lo];
      }
    jacobi_eigen(n, A, w, V);
    for (double x : w)
      if (!std::isfinite(x)) return PSOCI_ERR_NUMERIC;
    // ascending first (the order dsygv returns), then a stable sort to descending occupation
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return w[x] < w[y]; });
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return w[x] > w[y]; });
    for (int i = 0; i < n; ++i) {
      occ[eoff + i] = w[idx[i]];
      for (int k = 0; k < n; ++k) vecs[voff + (size_t)i * n + k] = V[(size_t)k * n + idx[i]];
    }
    eoff += n;
    voff += (size_t)n * n;
    b0 = b1;
  }
  return PSOCI_OK;
}
