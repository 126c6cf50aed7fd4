// evr_krylov.h -- host-side algebra of the short-iterative-Lanczos propagator: the
// propagator column u = exp(-i T t) e_1 of the Lanczos matrix T (symmetric tridiagonal,
// k <= a few hundred), from its eigen-decomposition, as UPsi_spec computes it
// (Source_ElVibRot/sub_propagation/sub_module_propa_march.f90:3101-3160).
// Header-only and free of CUDA so that it is compiled, unchanged, by the CPU tests.
#ifndef EVR_KRYLOV_H
#define EVR_KRYLOV_H

#include <cmath>
#include <vector>

namespace evr {

// Eigen-decomposition of the real symmetric n x n matrix A (column-major, overwritten) by
// cyclic Jacobi rotations (Jacobi's method: each rotation in the (p,q) plane annihilates
// A_pq; sweeps repeat until the off-diagonal part is below 1e-15 of the Frobenius norm).
// On return w[i] = A_ii holds the eigenvalues and V's columns the eigenvectors.
// Returns false if 100 sweeps did not converge.
inline bool sym_eig_jacobi(int n, std::vector<double>& A, std::vector<double>& w, std::vector<double>& V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  double fro = 0.0;
  for (double x : A) fro += x * x;
  fro = std::sqrt(fro);
  bool ok = false;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int q = 1; q < n; ++q)
      for (int p = 0; p < q; ++p) off += A[p + (size_t)n * q] * A[p + (size_t)n * q];
    if (std::sqrt(2.0 * off) <= 1e-15 * fro || fro == 0.0) { ok = true; break; }
    for (int q = 1; q < n; ++q)
      for (int p = 0; p < q; ++p) {
        const double apq = A[p + (size_t)n * q];
        if (apq == 0.0) continue;
        // tan of the angle that zeroes A_pq: t^2 + 2 theta t - 1 = 0, smaller root
        const double theta = (A[q + (size_t)n * q] - A[p + (size_t)n * p]) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int r = 0; r < n; ++r) {  // columns p, q of A J
          const double x = A[r + (size_t)n * p], y = A[r + (size_t)n * q];
          A[r + (size_t)n * p] = c * x - s * y;
          A[r + (size_t)n * q] = s * x + c * y;
        }
        for (int r = 0; r < n; ++r) {  // rows p, q of J^T (A J)
          const double x = A[p + (size_t)n * r], y = A[q + (size_t)n * r];
          A[p + (size_t)n * r] = c * x - s * y;
          A[q + (size_t)n * r] = s * x + c * y;
        }
        A[p + (size_t)n * q] = 0.0;
        A[q + (size_t)n * p] = 0.0;
        for (int r = 0; r < n; ++r) {  // V J
          const double x = V[r + (size_t)n * p], y = V[r + (size_t)n * q];
          V[r + (size_t)n * p] = c * x - s * y;
          V[r + (size_t)n * q] = s * x + c * y;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = A[i + (size_t)n * i];
  return ok;
}

// u = exp(-i T t) e_1 for the symmetric tridiagonal T of order n with diagonal a[0..n-1]
// and off-diagonal b[0..n-2]: u_j = sum_i V_ji V_0i exp(-i lambda_i t).
inline bool krylov_propagator_column(int n, const double* a, const double* b, double t, double* ure, double* uim) {
  std::vector<double> A((size_t)n * n, 0.0), w, V;
  for (int i = 0; i < n; ++i) A[i + (size_t)n * i] = a[i];
  for (int i = 0; i + 1 < n; ++i) A[i + 1 + (size_t)n * i] = A[i + (size_t)n * (i + 1)] = b[i];
  const bool ok = sym_eig_jacobi(n, A, w, V);
  for (int j = 0; j < n; ++j) {
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < n; ++i) {
      const double f = V[j + (size_t)n * i] * V[(size_t)n * i];
      sr += f * std::cos(w[i] * t);
      si -= f * std::sin(w[i] * t);
    }
    ure[j] = sr;
    uim[j] = si;
  }
  return ok;
}

}  // namespace evr

#endif  // EVR_KRYLOV_H
