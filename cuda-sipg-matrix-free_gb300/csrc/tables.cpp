// tables.cpp -- host construction of the per-degree operator tables.
//
// LGL nodes: the N-1 interior nodes are the roots of P'_N, found by Newton's
// method on q(x) = (1 - x^2) P'_N(x) (whose derivative is -N(N+1) P_N(x)),
// started from the Chebyshev-Gauss-Lobatto points -cos(pi k / N); the end
// points are -1 and 1.  Weights: w_k = 2 / (N (N+1) P_N(x_k)^2).  Derivative
// matrix of the nodal Lagrange basis at the nodes: D[i][k] = P_N(x_k) /
// (P_N(x_i) (x_k - x_i)) for i != k, D[0][0] = -N(N+1)/4, D[N][N] = N(N+1)/4,
// 0 otherwise (the same closed form as sem_function<T>::d_phi,
// sem_function.hpp:86-110).  K[a][b] = sum_k w_k D[a][k] D[b][k].
#include <cmath>
#include <cstring>

#include "sipg_internal.cuh"

namespace sipg {

namespace {

// P_N(x) and P'_N(x) by the three-term recurrence.
void legendre(int N, double x, double* P, double* dP) {
  double p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
  if (N == 0) {
    *P = 1.0;
    *dP = 0.0;
    return;
  }
  for (int n = 1; n < N; ++n) {
    const double p2 = ((2 * n + 1) * x * p1 - n * p0) / (n + 1);
    const double d2 = d0 + (2 * n + 1) * p1;  // P'_{n+1} = P'_{n-1} + (2n+1) P_n
    p0 = p1;
    p1 = p2;
    d0 = d1;
    d1 = d2;
  }
  *P = p1;
  *dP = d1;
}

}  // namespace

int lgl_compute(int N, double* x, double* w) {
  if (N < 1 || N > 63) return -1;
  const int n = N + 1;
  x[0] = -1.0;
  x[N] = 1.0;
  for (int k = 1; k < N; ++k) {
    double xk = -std::cos(M_PI * k / N);
    for (int it = 0; it < 100; ++it) {
      double P, dP;
      legendre(N, xk, &P, &dP);
      const double q = (1.0 - xk * xk) * dP;
      const double dq = -N * (N + 1) * P;
      const double dx = q / dq;
      xk -= dx;
      if (std::fabs(dx) <= 1e-17 * (1.0 + std::fabs(xk))) break;
    }
    x[k] = xk;
  }
  // exact symmetry and the centre node
  for (int k = 0; k < n / 2; ++k) {
    const double m = 0.5 * (x[N - k] - x[k]);
    x[k] = -m;
    x[N - k] = m;
  }
  if (N % 2 == 0) x[N / 2] = 0.0;
  for (int k = 0; k < n; ++k) {
    double P, dP;
    legendre(N, x[k], &P, &dP);
    w[k] = 2.0 / (N * (N + 1) * P * P);
  }
  return 0;
}

int dphi_compute(int N, const double* x, double* D) {
  if (N < 1 || N > 63) return -1;
  const int n = N + 1;
  double PN[64];
  for (int k = 0; k < n; ++k) {
    double dP;
    legendre(N, x[k], &PN[k], &dP);
  }
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) {
      double v;
      if (i == k)
        v = (k == 0) ? -0.25 * N * (N + 1) : (k == N ? 0.25 * N * (N + 1) : 0.0);
      else
        v = PN[k] / (PN[i] * (x[k] - x[i]));
      D[i * n + k] = v;
    }
  return 0;
}

int build_host_tables(int p, HostTables* t) {
  if (p < 1 || p > SIPG_MAX_P || !t) return -1;
  std::memset(t, 0, sizeof(*t));
  const int n = p + 1;
  t->p = p;
  lgl_compute(p, t->nodes, t->w);
  dphi_compute(p, t->nodes, t->D);
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += t->w[k] * t->D[a * n + k] * t->D[b * n + k];
      t->K[a * n + b] = s;
    }
  // K is symmetric: make it exactly so
  for (int a = 0; a < n; ++a)
    for (int b = a + 1; b < n; ++b) {
      const double m = 0.5 * (t->K[a * n + b] + t->K[b * n + a]);
      t->K[a * n + b] = t->K[b * n + a] = m;
    }
  return 0;
}

}  // namespace sipg
