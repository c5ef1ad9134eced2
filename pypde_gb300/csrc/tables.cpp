// tables.cpp -- host precompute of the constant tables of one order N
// (a13 of the hot path): scaled Gauss-Legendre nodes and weights, the
// Lagrange basis in the power form of the reference's poly class, DERVALS,
// ENDVALS, the inverses of the WENO stencil matrices, the oscillation
// indicator and the DG time matrix with its inverse.
//
// Follows haranjackson/PyPDE src/scipy/math/legendre.cpp:136-197 (leggauss:
// roots of P_N, one Newton step, Clenshaw-based weights, symmetrisation),
// src/poly/basis.cpp:7-76, src/solvers/weno/weno_matrices.cpp:8-51 and
// src/solvers/dg/dg_matrices.cpp:32-55 with dg.cpp:38-40.  For N <= 3 the
// tables are bit-identical to the reference's (checked by the tests against
// vectors produced by the reference itself); for larger N the GL weights
// may differ from the reference's in the last few bits because the
// reference starts its Newton step from Eigen's companion-matrix
// eigenvalues.
#include "runtime.h"

#include <cmath>
#include <cstring>

namespace pypde {
namespace {

struct Poly {
  int n = 0;
  double c[2 * MAXN + 2];
};

double peval(const Poly &p, double x) {
  double r = 0;
  for (int i = 0; i < p.n; i++)
    r += p.c[i] * std::pow(x, (double)i);
  return r;
}
Poly pdiff1(const Poly &p) {
  Poly r;
  r.n = p.n - 1;
  for (int i = 0; i < r.n; i++)
    r.c[i] = p.c[i + 1] * (i + 1);
  return r;
}
Poly pdiff(Poly p, int k) {
  for (int i = 0; i < k; i++)
    p = pdiff1(p);
  return p;
}
Poly pint(const Poly &p) {
  Poly r;
  r.n = p.n + 1;
  r.c[0] = 0;
  for (int i = 1; i < r.n; i++)
    r.c[i] = p.c[i - 1] / i;
  return r;
}
Poly pmul(const Poly &a, const Poly &b) {
  Poly r;
  r.n = a.n + b.n - 1;
  for (int i = 0; i < r.n; i++)
    r.c[i] = 0;
  for (int i = 0; i < a.n; i++)
    for (int j = 0; j < b.n; j++)
      r.c[i + j] += a.c[i] * b.c[j];
  return r;
}

// Clenshaw evaluation of a Legendre series (legendre.cpp:5-60)
double legval(double x, const double *c, int nc) {
  if (nc == 1)
    return c[0];
  if (nc == 2)
    return c[0] + c[1] * x;
  int nd = nc - 1;
  double c0 = c[nc - 3] - (c[nc - 1] * (nd - 1)) / nd;
  double c1 = c[nc - 2] + (c[nc - 1] * x * (2 * nd - 1)) / nd;
  if (nc == 3)
    return c0 + c1 * x;
  nd -= 1;
  double c00 = c[nc - 4] - (c1 * (nd - 1)) / nd;
  double c11 = c0 + (c1 * x * (2 * nd - 1)) / nd;
  for (int i = 5; i < nc + 1; i++) {
    double tmp = c00;
    nd -= 1;
    c00 = c[nc - i] - (c11 * (nd - 1)) / nd;
    c11 = tmp + (c11 * x * (2 * nd - 1)) / nd;
  }
  return c00 + c11 * x;
}

// Legendre-series derivative (legendre.cpp:96-134)
void legder(const double *cin, int nc, double *der) {
  double c[MAXN + 2];
  int n = nc - 1;
  std::memcpy(c, cin, sizeof(double) * nc);
  for (int j = 0; j < n; j++)
    der[j] = 0;
  for (int j = n; j > 2; j--) {
    der[j - 1] = (2 * j - 1) * c[j];
    c[j - 2] += c[j];
  }
  if (n > 1)
    der[1] = 3 * c[2];
  der[0] = c[1];
}

void gauss_legendre(int deg, double *x, double *w) {
  double c[MAXN + 2], dc[MAXN + 2];
  for (int i = 0; i <= deg; i++)
    c[i] = 0;
  c[deg] = 1;
  legder(c, deg + 1, dc);
  for (int k = 0; k < deg; k++) {
    double r = -std::cos(M_PI * (k + 0.75) / (deg + 0.5));
    for (int it = 0; it < 100; it++) {
      double dr = legval(r, c, deg + 1) / legval(r, dc, deg);
      r -= dr;
      if (std::fabs(dr) <= 1e-17)
        break;
    }
    x[k] = r;
  }
  double df[MAXN], fm[MAXN];
  for (int k = 0; k < deg; k++) {
    double dy = legval(x[k], c, deg + 1);
    df[k] = legval(x[k], dc, deg);
    x[k] -= dy / df[k];
  }
  double fmax_ = 0, dmax = 0;
  for (int k = 0; k < deg; k++) {
    fm[k] = legval(x[k], c + 1, deg);
    fmax_ = std::fmax(fmax_, std::fabs(fm[k]));
    dmax = std::fmax(dmax, std::fabs(df[k]));
  }
  double ws[MAXN], xs[MAXN], sum = 0;
  for (int k = 0; k < deg; k++)
    ws[k] = 1. / ((fm[k] / fmax_) * (df[k] / dmax));
  for (int k = 0; k < deg; k++) {
    w[k] = (ws[k] + ws[deg - 1 - k]) / 2;
    xs[k] = (x[k] - x[deg - 1 - k]) / 2;
  }
  for (int k = 0; k < deg; k++) {
    x[k] = xs[k];
    sum += w[k];
  }
  for (int k = 0; k < deg; k++)
    w[k] *= 2. / sum;
}

int invert(const double *a, int n, double *inv) {
  double m[MAXN][2 * MAXN];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      m[i][j] = a[i * n + j];
      m[i][n + j] = (i == j) ? 1.0 : 0.0;
    }
  for (int col = 0; col < n; col++) {
    int piv = col;
    for (int r = col + 1; r < n; r++)
      if (std::fabs(m[r][col]) > std::fabs(m[piv][col]))
        piv = r;
    if (m[piv][col] == 0.0)
      return -1;
    if (piv != col)
      for (int j = 0; j < 2 * n; j++)
        std::swap(m[col][j], m[piv][j]);
    double p = m[col][col];
    for (int j = 0; j < 2 * n; j++)
      m[col][j] /= p;
    for (int r = 0; r < n; r++)
      if (r != col && m[r][col] != 0.0) {
        double f = m[r][col];
        for (int j = 0; j < 2 * n; j++)
          m[r][j] -= f * m[col][j];
      }
  }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      inv[i * n + j] = m[i][n + j];
  return 0;
}

} // namespace

int make_tables(int N, Tables *T) {
  if (N < 1 || N > MAXN)
    return -1;
  std::memset(T, 0, sizeof(*T));
  T->N = N;
  double x[MAXN], w[MAXN];
  gauss_legendre(N, x, w);
  for (int i = 0; i < N; i++) {
    T->nodes[i] = (x[i] + 1) / 2;
    T->wghts[i] = w[i] / 2;
  }
  Poly psi[MAXN];
  for (int i = 0; i < N; i++) {
    Poly p;
    p.n = 1;
    p.c[0] = 1.0;
    for (int j = 0; j < N; j++) {
      if (j == i)
        continue;
      Poly q;
      q.n = 2;
      q.c[0] = -T->nodes[j];
      q.c[1] = 1.0;
      p = pmul(p, q);
      double den = T->nodes[i] - T->nodes[j];
      for (int k = 0; k < p.n; k++)
        p.c[k] /= den;
    }
    psi[i] = p;
  }
  for (int j = 0; j < N; j++) {
    T->endvals[j] = peval(psi[j], 0.);
    T->endvals[N + j] = peval(psi[j], 1.);
  }
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      T->dervals[i * N + j] = peval(pdiff(psi[j], 1), T->nodes[i]);
  int FN2 = (int)std::floor((N - 1) / 2.), CN2 = (int)std::ceil((N - 1) / 2.);
  double m[4][MAXN * MAXN];
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      Poly P = pint(psi[j]);
      m[0][i * N + j] = peval(P, i - N + 2) - peval(P, i - N + 1);
      m[1][i * N + j] = peval(P, i + 1) - peval(P, i);
      m[2][i * N + j] = peval(P, i - CN2 + 1) - peval(P, i - CN2);
      m[3][i * N + j] = peval(P, i - FN2 + 1) - peval(P, i - FN2);
    }
  for (int k = 0; k < 4; k++)
    invert(m[k], N, T->weno_inv[k]);
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      double s = 0;
      for (int a = 1; a < N; a++) {
        Poly P = pint(pmul(pdiff(psi[i], a), pdiff(psi[j], a)));
        s += peval(P, 1) - peval(P, 0);
      }
      T->sig[i * N + j] = s;
    }
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      double end = peval(psi[i], 1) * peval(psi[j], 1);
      double der;
      if (i == j) {
        double e0 = peval(psi[j], 0), e1 = peval(psi[j], 1);
        der = (e1 * e1 - e0 * e0) / 2;
      } else {
        der = T->wghts[j] * peval(pdiff(psi[i], 1), T->nodes[j]);
      }
      T->dgmat[i * N + j] = end - der;
    }
  invert(T->dgmat, N, T->dgmat_inv);
  return 0;
}

void make_wprod(const Tables &T, int ndim, double *wprod) {
  int N = T.N, Nd = 1;
  for (int d = 0; d < ndim; d++)
    Nd *= N;
  for (int idx = 0; idx < Nd; idx++) {
    int digs[3] = {0, 0, 0}, r = idx;
    for (int d = ndim - 1; d >= 0; d--) {
      digs[d] = r % N;
      r /= N;
    }
    double p = 1.0;
    for (int d = 0; d < ndim; d++)
      p *= T.wghts[digs[d]];
    wprod[idx] = p;
  }
}

} // namespace pypde
