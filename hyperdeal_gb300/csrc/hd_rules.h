// hd_rules.h -- one-dimensional quadrature rules and Lagrange tables on [0,1],
// shared by the host code of every entry point (hd_capi.cu, hd_noalloc.cu).
//
// deal.II (a dependency of the reference, not part of its tree) supplies these
// through QGaussLobatto / QGauss and the FE_DGQ shape data; here they are
// computed from the Legendre three-term recurrence and Newton's method.
#pragma once

#include <cmath>

namespace hd {
namespace rules {

// Legendre P_n and P_n' (three-term recurrence)
inline void legendre(int n, double x, double* p, double* dp) {
  double p0 = 1.0, p1 = x;
  if (n == 0) { *p = 1.0; *dp = 0.0; return; }
  for (int k = 2; k <= n; ++k) {
    const double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = pk;
  }
  *p = p1;
  *dp = n * (p0 - x * p1) / (1.0 - x * x);
}

// Gauss-Lobatto rule with n points on [0,1]: end points plus the roots of
// P_{n-1}' (Newton from Chebyshev-Gauss-Lobatto guesses); w = 2/(n(n-1)P^2)/2
inline void gauss_lobatto(int n, double* x, double* w) {
  const int m = n - 1;
  x[0] = 0.0;
  x[n - 1] = 1.0;
  for (int i = 1; i < m; ++i) {
    double z = -std::cos(M_PI * i / m);
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre(m, z, &p, &dp);
      const double ddp = (2.0 * z * dp - m * (m + 1.0) * p) / (1.0 - z * z);
      const double dz = dp / ddp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    x[i] = 0.5 * (1.0 + z);
  }
  for (int i = 0; i < n; ++i) {
    double p, dp;
    const double z = 2.0 * x[i] - 1.0;
    if (i == 0 || i == n - 1) {
      p = (i == 0 && (m % 2)) ? -1.0 : 1.0;  // P_m(+-1) = (+-1)^m
    } else {
      legendre(m, z, &p, &dp);
    }
    w[i] = 1.0 / (m * (m + 1.0) * p * p);
  }
  for (int i = 0; i < n / 2; ++i) {  // exact symmetry
    const double xs = 0.5 * (x[i] + (1.0 - x[n - 1 - i]));
    const double ws = 0.5 * (w[i] + w[n - 1 - i]);
    x[i] = xs;
    x[n - 1 - i] = 1.0 - xs;
    w[i] = ws;
    w[n - 1 - i] = ws;
  }
  if (n % 2) x[n / 2] = 0.5;
}

// D[q][j] = l_j'(x_q) for the Lagrange basis on the nodes x
inline void lagrange_derivative_matrix(int n, const double* x, double* D) {
  for (int q = 0; q < n; ++q)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int l = 0; l < n; ++l) {
        if (l == j) continue;
        double t = 1.0 / (x[j] - x[l]);
        for (int m = 0; m < n; ++m)
          if (m != j && m != l) t *= (x[q] - x[m]) / (x[j] - x[m]);
        s += t;
      }
      D[q * n + j] = s;
    }
}

// Gauss rule with n points on [0,1]: roots of P_n (Newton), w = 1/((1-z^2) P_n'(z)^2)
inline void gauss_rule(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    double p = 0.0, dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      legendre(n, z, &p, &dp);
      const double dz = p / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    legendre(n, z, &p, &dp);
    x[n - 1 - i] = 0.5 * (1.0 + z);
    w[n - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
  for (int i = 0; i < n / 2; ++i) {  // exact symmetry
    const double xs = 0.5 * (x[i] + (1.0 - x[n - 1 - i]));
    const double ws = 0.5 * (w[i] + w[n - 1 - i]);
    x[i] = xs;
    x[n - 1 - i] = 1.0 - xs;
    w[i] = ws;
    w[n - 1 - i] = ws;
  }
  if (n % 2) x[n / 2] = 0.5;
}

// L_j(t) of the Lagrange basis on the nodes x
inline double lagrange_value(int n, const double* x, int j, double t) {
  double v = 1.0;
  for (int m = 0; m < n; ++m)
    if (m != j) v *= (t - x[m]) / (x[j] - x[m]);
  return v;
}

}  // namespace rules
}  // namespace hd
