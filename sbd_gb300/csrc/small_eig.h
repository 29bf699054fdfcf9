// Dense symmetric eigensolvers for the projected (Rayleigh-Ritz) matrices of
// the Davidson solvers, n <= 64, FP64 on the host.  They stand in for the
// LAPACK dsyev call of the reference (framework/hp_numeric.h:503-520):
// eigenvalues ascending, eigenvectors in the columns.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

namespace sbdgb {

// Cyclic Jacobi.  A: n x n column-major (copied); w ascending; V column-major.
inline void jacobi_eig(int n, std::vector<double> A, std::vector<double> &w, std::vector<double> &Vout) {
  std::vector<double> V((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i + (size_t)n * i] = 1.0;
  auto a = [&](int i, int j) -> double & { return A[i + (size_t)n * j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, dg = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) (i == j ? dg : off) += a(i, j) * a(i, j);
    if (off <= 1e-30 * (dg + 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a(p, q);
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (a(q, q) - a(p, p)) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a(k, p), akq = a(k, q);
          a(k, p) = c * akp - s * akq;
          a(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a(p, k), aqk = a(q, k);
          a(p, k) = c * apk - s * aqk;
          a(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[k + (size_t)n * p], vkq = V[k + (size_t)n * q];
          V[k + (size_t)n * p] = c * vkp - s * vkq;
          V[k + (size_t)n * q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
  w.resize(n);
  Vout.assign((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    w[j] = a(idx[j], idx[j]);
    for (int i = 0; i < n; ++i) Vout[i + (size_t)n * j] = V[i + (size_t)n * idx[j]];
  }
}

// Generalized problem A v = w S v with S symmetric positive definite: Cholesky
// S = L L^T, eigenpairs of L^-1 A L^-T, v = L^-T y (so V^T S V = I).  Returns
// false if S is not numerically positive definite.
inline bool gen_sym_eig(int n, const std::vector<double> &A, const std::vector<double> &S, std::vector<double> &w,
                        std::vector<double> &V) {
  std::vector<double> L((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    double d = S[j + (size_t)n * j];
    for (int k = 0; k < j; ++k) d -= L[j + (size_t)n * k] * L[j + (size_t)n * k];
    if (!(d > 1e-14)) return false;
    const double ljj = std::sqrt(d);
    L[j + (size_t)n * j] = ljj;
    for (int i = j + 1; i < n; ++i) {
      double s = S[i + (size_t)n * j];
      for (int k = 0; k < j; ++k) s -= L[i + (size_t)n * k] * L[j + (size_t)n * k];
      L[i + (size_t)n * j] = s / ljj;
    }
  }
  // B = L^-1 A (forward substitution on every column)
  std::vector<double> B(A);
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < n; ++i) {
      double s = B[i + (size_t)n * c];
      for (int k = 0; k < i; ++k) s -= L[i + (size_t)n * k] * B[k + (size_t)n * c];
      B[i + (size_t)n * c] = s / L[i + (size_t)n * i];
    }
  // Cm = B L^-T = (L^-1 B^T)^T
  std::vector<double> Bt((size_t)n * n), Cm((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Bt[i + (size_t)n * j] = B[j + (size_t)n * i];
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < n; ++i) {
      double s = Bt[i + (size_t)n * c];
      for (int k = 0; k < i; ++k) s -= L[i + (size_t)n * k] * Bt[k + (size_t)n * c];
      Bt[i + (size_t)n * c] = s / L[i + (size_t)n * i];
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Cm[i + (size_t)n * j] = 0.5 * (Bt[j + (size_t)n * i] + Bt[i + (size_t)n * j]);
  std::vector<double> Y;
  jacobi_eig(n, Cm, w, Y);
  // V = L^-T Y (back substitution)
  V.assign((size_t)n * n, 0.0);
  for (int c = 0; c < n; ++c)
    for (int i = n - 1; i >= 0; --i) {
      double s = Y[i + (size_t)n * c];
      for (int k = i + 1; k < n; ++k) s -= L[k + (size_t)n * i] * V[k + (size_t)n * c];
      V[i + (size_t)n * c] = s / L[i + (size_t)n * i];
    }
  return true;
}

}  // namespace sbdgb
