// Eigen-decomposition of the small symmetric tridiagonal Lanczos matrix
// (n <= mlanc, a handful), the role LAPACK dstev plays in
// lanczos_su2::diatridiag (lanczos_su2.cpp:237-259).  Cyclic Jacobi rotations
// on the dense matrix (Golub & Van Loan, "Matrix Computations", sec. 8.5):
// unconditionally convergent and accurate to a few ulps of the matrix norm for
// these sizes.  Eigenvalues ascending; eigenvectors column-major in z
// (column j belongs to eigenvalue j), each of unit length.  Column signs,
// which dstev leaves to the LAPACK build, follow canonical_column_signs.
#pragma once
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace su2g {

// Sign rule for eigenvectors: in each column of the rows x cols matrix z
// (column-major, leading dimension ld) the first entry whose magnitude exceeds
// 1e-4 of the column's largest is made positive.  The reference takes the
// signs LAPACK happens to return; fixing them makes results independent of
// the eigen-solver (the svd's device eigenvectors follow the same rule).
inline void canonical_column_signs(int rows, int cols, double* z, int ld) {
  for (int c = 0; c < cols; ++c) {
    double* col = z + (size_t)c * ld;
    double mx = 0;
    for (int i = 0; i < rows; ++i) mx = std::max(mx, std::fabs(col[i]));
    for (int i = 0; i < rows; ++i)
      if (std::fabs(col[i]) > 1e-4 * mx) {
        if (col[i] < 0)
          for (int k = 0; k < rows; ++k) col[k] = -col[k];
        break;
      }
  }
}

inline void tridiag_eigh(const std::vector<double>& d, const std::vector<double>& e, std::vector<double>* w,
                         std::vector<double>* z) {
  const int n = (int)d.size();
  std::vector<double> a(n * n, 0.0), v(n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    a[i + i * n] = d[i];
    v[i + i * n] = 1.0;
    if (i + 1 < n) a[i + (i + 1) * n] = a[(i + 1) + i * n] = e[i];
  }
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, norm = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        norm += a[i + j * n] * a[i + j * n];
        if (i != j) off += a[i + j * n] * a[i + j * n];
      }
    if (off <= 1e-36 * norm || off == 0) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[p + q * n];
        if (apq == 0) continue;
        const double app = a[p + p * n], aqq = a[q + q * n];
        const double theta = (aqq - app) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        const double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- A J (columns p, q)
          const double akp = a[k + p * n], akq = a[k + q * n];
          a[k + p * n] = c * akp - s * akq;
          a[k + q * n] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // A <- J^T A (rows p, q)
          const double apk = a[p + k * n], aqk = a[q + k * n];
          a[p + k * n] = c * apk - s * aqk;
          a[q + k * n] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {  // V <- V J
          const double vkp = v[k + p * n], vkq = v[k + q * n];
          v[k + p * n] = c * vkp - s * vkq;
          v[k + q * n] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return a[x + x * n] < a[y + y * n]; });
  w->assign(n, 0.0);
  z->assign(n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    (*w)[j] = a[order[j] + order[j] * n];
    for (int i = 0; i < n; ++i) (*z)[i + j * n] = v[i + order[j] * n];
  }
  canonical_column_signs(n, n, z->data(), n);
}

}  // namespace su2g
