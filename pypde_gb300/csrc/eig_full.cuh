// eig_full.cuh -- full real eigen-decomposition for the Roe and Osher
// fluxes (a11, fluxes.cpp:20-70): Householder Hessenberg reduction with the
// orthogonal factor accumulated, Francis double-shift QR to real Schur form
// with Schur vectors, eigenvectors by back substitution on the
// quasi-triangular factor (V = Z X), and a complex LU solve with partial
// pivoting.  Statement for statement the host restatement's ora_eig and
// csolve (Golub & Van Loan, Alg. 7.4.2, 7.5.1, 7.6.x), so both give the same
// bits.  Replaces Eigen::EigenSolver and colPivHouseholderQr.
#pragma once

#include "ader_common.cuh"

namespace pypde {

#define A_(i, j) a[(i) * n + (j)]

template <int V>
__device__ __noinline__ void hessenberg_q(double *a, double *q) {
  const int n = V;
  if (q)
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        q[i * n + j] = (i == j);
  for (int k = 0; k < n - 2; k++) {
    double v[V], alpha = 0, scale = 0;
    for (int i = k + 1; i < n; i++)
      scale += fabs(A_(i, k));
    if (scale == 0.0)
      continue;
    for (int i = k + 1; i < n; i++) {
      v[i] = A_(i, k) / scale;
      alpha += v[i] * v[i];
    }
    double g = sqrt(alpha);
    if (v[k + 1] > 0)
      g = -g;
    double h = alpha - v[k + 1] * g; /* = |v|^2 / 2 after v[k+1] -= g */
    v[k + 1] -= g;
    /* A <- P A, P = I - v v^T / h */
    for (int j = k; j < n; j++) {
      double s = 0;
      for (int i = k + 1; i < n; i++)
        s += v[i] * A_(i, j);
      s /= h;
      for (int i = k + 1; i < n; i++)
        A_(i, j) -= s * v[i];
    }
    /* A <- A P */
    for (int i = 0; i < n; i++) {
      double s = 0;
      for (int j = k + 1; j < n; j++)
        s += A_(i, j) * v[j];
      s /= h;
      for (int j = k + 1; j < n; j++)
        A_(i, j) -= s * v[j];
    }
    if (q)
      for (int i = 0; i < n; i++) {
        double s = 0;
        for (int j = k + 1; j < n; j++)
          s += q[i * n + j] * v[j];
        s /= h;
        for (int j = k + 1; j < n; j++)
          q[i * n + j] -= s * v[j];
      }
    A_(k + 1, k) = g * scale;
    for (int i = k + 2; i < n; i++)
      A_(i, k) = 0.0;
  }
}


template <int V>
__device__ __noinline__ int francis_full(double *a, double *wr, double *wi,
                                              int wantt, double *z) {
  const int n = V;
  double norm = 0;
  for (int i = 0; i < n; i++)
    for (int j = (i > 0 ? i - 1 : 0); j < n; j++)
      norm += fabs(A_(i, j));
  int hi = n - 1, its = 0, total = 0;
  double exshift = 0.0;
  while (hi >= 0) {
    int l;
    for (l = hi; l > 0; l--) { /* deflation */
      double s = fabs(A_(l - 1, l - 1)) + fabs(A_(l, l));
      if (s == 0.0)
        s = norm;
      if (fabs(A_(l, l - 1)) <= DBL_EPS * s) {
        A_(l, l - 1) = 0.0;
        break;
      }
    }
    if (l == hi) { /* 1x1 block */
      wr[hi] = A_(hi, hi) + exshift;
      wi[hi] = 0.0;
      if (wantt)
        A_(hi, hi) = wr[hi];
      hi--;
      its = 0;
      continue;
    }
    if (l == hi - 1) { /* 2x2 block */
      double p = 0.5 * (A_(hi - 1, hi - 1) - A_(hi, hi));
      double qq = p * p + A_(hi, hi - 1) * A_(hi - 1, hi);
      double zz = sqrt(fabs(qq));
      double x = A_(hi, hi) + exshift;
      if (wantt) {
        A_(hi, hi) += exshift;
        A_(hi - 1, hi - 1) += exshift;
      }
      if (qq >= 0.0) { /* real pair */
        zz = (p >= 0) ? p + zz : p - zz;
        wr[hi - 1] = x + zz;
        wr[hi] = (zz != 0.0) ? x - A_(hi, hi - 1) * A_(hi - 1, hi) / zz
                             : x + zz;
        wi[hi - 1] = wi[hi] = 0.0;
        if (wantt) { /* rotate the block to upper triangular form */
          double xx = A_(hi, hi - 1);
          double s = fabs(xx) + fabs(zz);
          double pp = xx / s, q2 = zz / s;
          double r = sqrt(pp * pp + q2 * q2);
          pp /= r;
          q2 /= r;
          for (int j = hi - 1; j < n; j++) {
            double t = A_(hi - 1, j);
            A_(hi - 1, j) = q2 * t + pp * A_(hi, j);
            A_(hi, j) = q2 * A_(hi, j) - pp * t;
          }
          for (int i = 0; i <= hi; i++) {
            double t = A_(i, hi - 1);
            A_(i, hi - 1) = q2 * t + pp * A_(i, hi);
            A_(i, hi) = q2 * A_(i, hi) - pp * t;
          }
          if (z)
            for (int i = 0; i < n; i++) {
              double t = z[i * n + hi - 1];
              z[i * n + hi - 1] = q2 * t + pp * z[i * n + hi];
              z[i * n + hi] = q2 * z[i * n + hi] - pp * t;
            }
          A_(hi, hi - 1) = 0.0;
          A_(hi - 1, hi - 1) = wr[hi - 1];
          A_(hi, hi) = wr[hi];
        }
      } else { /* complex pair */
        wr[hi - 1] = wr[hi] = x + p;
        wi[hi - 1] = zz;
        wi[hi] = -zz;
      }
      hi -= 2;
      its = 0;
      continue;
    }
    /* shifts */
    double x = A_(hi, hi), y = A_(hi - 1, hi - 1);
    double w = A_(hi, hi - 1) * A_(hi - 1, hi);
    if (its == 10 || its == 20) { /* exceptional shift */
      exshift += x;
      for (int i = 0; i <= hi; i++)
        A_(i, i) -= x;
      double s = fabs(A_(hi, hi - 1)) + fabs(A_(hi - 1, hi - 2));
      x = y = 0.75 * s;
      w = -0.4375 * s * s;
    }
    its++;
    if (++total > 40 * n)
      return -1;
    /* look for two consecutive small subdiagonals (start row m) */
    int m;
    double p = 0, q = 0, r = 0;
    for (m = hi - 2; m >= l; m--) {
      double zz = A_(m, m);
      double rr = x - zz, ss = y - zz;
      p = (rr * ss - w) / A_(m + 1, m) + A_(m, m + 1);
      q = A_(m + 1, m + 1) - zz - rr - ss;
      r = A_(m + 2, m + 1);
      double s = fabs(p) + fabs(q) + fabs(r);
      p /= s;
      q /= s;
      r /= s;
      if (m == l)
        break;
      double u = fabs(A_(m, m - 1)) * (fabs(q) + fabs(r));
      double vv = fabs(p) * (fabs(A_(m - 1, m - 1)) + fabs(zz) +
                             fabs(A_(m + 1, m + 1)));
      if (u <= DBL_EPS * vv)
        break;
    }
    for (int i = m + 2; i <= hi; i++) {
      A_(i, i - 2) = 0.0;
      if (i > m + 2)
        A_(i, i - 3) = 0.0;
    }
    /* double-shift sweep rows/cols m..hi */
    for (int k = m; k <= hi - 1; k++) {
      int notlast = (k != hi - 1);
      if (k != m) {
        p = A_(k, k - 1);
        q = A_(k + 1, k - 1);
        r = notlast ? A_(k + 2, k - 1) : 0.0;
        x = fabs(p) + fabs(q) + fabs(r);
        if (x == 0.0)
          continue;
        p /= x;
        q /= x;
        r /= x;
      }
      double s = sqrt(p * p + q * q + r * r);
      if (p < 0)
        s = -s;
      if (k != m)
        A_(k, k - 1) = -s * x;
      else if (l != m)
        A_(k, k - 1) = -A_(k, k - 1);
      p += s;
      x = p / s;
      y = q / s;
      double zz = r / s;
      q /= p;
      r /= p;
      int jlo = k, jhi = wantt ? n - 1 : hi;
      for (int j = jlo; j <= jhi; j++) { /* row update */
        double pp = A_(k, j) + q * A_(k + 1, j);
        if (notlast) {
          pp += r * A_(k + 2, j);
          A_(k + 2, j) -= pp * zz;
        }
        A_(k + 1, j) -= pp * y;
        A_(k, j) -= pp * x;
      }
      int ilo = wantt ? 0 : l;
      int ihi = (hi < k + 3) ? hi : k + 3;
      for (int i = ilo; i <= ihi; i++) { /* column update */
        double pp = x * A_(i, k) + y * A_(i, k + 1);
        if (notlast) {
          pp += zz * A_(i, k + 2);
          A_(i, k + 2) -= pp * r;
        }
        A_(i, k + 1) -= pp * q;
        A_(i, k) -= pp;
      }
      if (z)
        for (int i = 0; i < n; i++) {
          double pp = x * z[i * n + k] + y * z[i * n + k + 1];
          if (notlast) {
            pp += zz * z[i * n + k + 2];
            z[i * n + k + 2] -= pp * r;
          }
          z[i * n + k + 1] -= pp * q;
          z[i * n + k] -= pp;
        }
    }
  }
  return 0;
}


template <int V>
__device__ __noinline__ int eig_full(const double *ain, double *wr, double *wi,
                                          double *vr, double *vi) {
  const int n = V;
  double a[V * V], z[V * V];
  for (int i_ = 0; i_ < n * n; i_++)
    a[i_] = ain[i_];
  hessenberg_q<V>(a, z);
  if (francis_full<V>(a, wr, wi, 1, z) != 0)
    return -1;
  double norm = 0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      norm += fabs(A_(i, j));
  double smin = DBL_EPS * (norm > 0 ? norm : 1.0);
  double xr[V], xi[V];
  for (int k = 0; k < n; k++) {
    double lr = wr[k], li = wi[k];
    for (int i = 0; i < n; i++)
      xr[i] = xi[i] = 0.0;
    int top;
    if (li == 0.0) {
      xr[k] = 1.0;
      top = k - 1;
    } else if (li > 0.0) { /* first of a pair: block (k, k+1) */
      /* eigenvector of the 2x2 block [[a b],[c d]] for lambda = lr + i li:
       * x_{k+1} = 1, x_k = (lambda - d) / c ... use the row with larger
       * coefficient for stability */
      double b = A_(k, k + 1), c = A_(k + 1, k);
      if (fabs(b) >= fabs(c)) {
        xr[k] = 1.0;
        xi[k] = 0.0;
        /* (a - lambda) x_k + b x_{k+1} = 0 */
        xr[k + 1] = -(A_(k, k) - lr) / b;
        xi[k + 1] = li / b;
      } else {
        xr[k + 1] = 1.0;
        xi[k + 1] = 0.0;
        /* c x_k + (d - lambda) x_{k+1} = 0 */
        xr[k] = -(A_(k + 1, k + 1) - lr) / c;
        xi[k] = li / c;
      }
      top = k - 1;
    } else { /* second of a pair: conjugate of the first */
      for (int i = 0; i < n; i++) {
        vr[i * n + k] = vr[i * n + k - 1];
        vi[i * n + k] = -vi[i * n + k - 1];
      }
      continue;
    }
    int last = (li > 0.0) ? k + 1 : k;
    for (int i = top; i >= 0; i--) {
      int blk2 = (i > 0 && A_(i, i - 1) != 0.0);
      if (!blk2) {
        double sr = 0, si = 0;
        for (int j = i + 1; j <= last; j++) {
          sr += A_(i, j) * xr[j];
          si += A_(i, j) * xi[j];
        }
        double dr = A_(i, i) - lr, di = -li;
        if (fabs(dr) + fabs(di) < smin)
          dr = smin;
        double den = dr * dr + di * di; /* x = -s / (dr + i di) */
        xr[i] = -(sr * dr + si * di) / den;
        xi[i] = -(si * dr - sr * di) / den;
      } else { /* 2x2 block rows i-1, i */
        double s1r = 0, s1i = 0, s2r = 0, s2i = 0;
        for (int j = i + 1; j <= last; j++) {
          s1r += A_(i - 1, j) * xr[j];
          s1i += A_(i - 1, j) * xi[j];
          s2r += A_(i, j) * xr[j];
          s2i += A_(i, j) * xi[j];
        }
        /* [[a-l, b],[c, d-l]] [x1;x2] = -[s1; s2], complex l */
        double ar = A_(i - 1, i - 1) - lr, ai = -li, b = A_(i - 1, i);
        double c = A_(i, i - 1), dr = A_(i, i) - lr, di = -li;
        /* det = (ar + i ai)(dr + i di) - b c */
        double detr = ar * dr - ai * di - b * c, deti = ar * di + ai * dr;
        if (fabs(detr) + fabs(deti) < smin)
          detr = smin;
        double dd = detr * detr + deti * deti;
        /* x1 = (-(d-l) s1 + b s2) / det ; x2 = (c s1 - (a-l) s2) / det */
        double n1r = -(dr * s1r - di * s1i) + b * s2r;
        double n1i = -(dr * s1i + di * s1r) + b * s2i;
        double n2r = c * s1r - (ar * s2r - ai * s2i);
        double n2i = c * s1i - (ar * s2i + ai * s2r);
        xr[i - 1] = (n1r * detr + n1i * deti) / dd;
        xi[i - 1] = (n1i * detr - n1r * deti) / dd;
        xr[i] = (n2r * detr + n2i * deti) / dd;
        xi[i] = (n2i * detr - n2r * deti) / dd;
        i--;
      }
    }
    /* v = Z x, normalised to unit 2-norm */
    double nrm = 0;
    for (int i = 0; i < n; i++) {
      double sr = 0, si = 0;
      for (int j = 0; j <= last; j++) {
        sr += z[i * n + j] * xr[j];
        si += z[i * n + j] * xi[j];
      }
      vr[i * n + k] = sr;
      vi[i * n + k] = si;
      nrm += sr * sr + si * si;
    }
    nrm = sqrt(nrm);
    for (int i = 0; i < n; i++) {
      vr[i * n + k] /= nrm;
      vi[i * n + k] /= nrm;
    }
  }
  return 0;
}
#undef A_

template <int V>
__device__ __noinline__ int csolve(double *mr, double *mi, double *br, double *bi) {
  const int n = V;
  for (int c = 0; c < n; c++) {
    int piv = c;
    double best = sqrt(mr[c * n + c] * mr[c * n + c] + mi[c * n + c] * mi[c * n + c]);
    for (int r = c + 1; r < n; r++) {
      double v = sqrt(mr[r * n + c] * mr[r * n + c] + mi[r * n + c] * mi[r * n + c]);
      if (v > best) {
        best = v;
        piv = r;
      }
    }
    if (best == 0.0)
      return -1;
    if (piv != c) {
      for (int j = 0; j < n; j++) {
        double t = mr[c * n + j];
        mr[c * n + j] = mr[piv * n + j];
        mr[piv * n + j] = t;
        t = mi[c * n + j];
        mi[c * n + j] = mi[piv * n + j];
        mi[piv * n + j] = t;
      }
      double t = br[c];
      br[c] = br[piv];
      br[piv] = t;
      t = bi[c];
      bi[c] = bi[piv];
      bi[piv] = t;
    }
    double pr = mr[c * n + c], pi = mi[c * n + c], pd = pr * pr + pi * pi;
    for (int r = c + 1; r < n; r++) {
      double fr = (mr[r * n + c] * pr + mi[r * n + c] * pi) / pd;
      double fi = (mi[r * n + c] * pr - mr[r * n + c] * pi) / pd;
      for (int j = c; j < n; j++) {
        mr[r * n + j] -= fr * mr[c * n + j] - fi * mi[c * n + j];
        mi[r * n + j] -= fr * mi[c * n + j] + fi * mr[c * n + j];
      }
      br[r] -= fr * br[c] - fi * bi[c];
      bi[r] -= fr * bi[c] + fi * br[c];
    }
  }
  for (int r = n - 1; r >= 0; r--) {
    double sr = br[r], si = bi[r];
    for (int j = r + 1; j < n; j++) {
      sr -= mr[r * n + j] * br[j] - mi[r * n + j] * bi[j];
      si -= mr[r * n + j] * bi[j] + mi[r * n + j] * br[j];
    }
    double pr = mr[r * n + r], pi = mi[r * n + r], pd = pr * pr + pi * pi;
    br[r] = (sr * pr + si * pi) / pd;
    bi[r] = (si * pr - sr * pi) / pd;
  }
  return 0;
}


} // namespace pypde
