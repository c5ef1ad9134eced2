// ader_common.cuh -- constants, per-(ndim,N) tables and the FP64 numerics
// shared by the ADER-WENO kernels.
//
// Plain-form arithmetic is bit-faithful to the reference algorithm as
// restated on the host (cited per function; paths relative to
// haranjackson/PyPDE).  The translation units are compiled with
// --fmad=false so that no multiply-add is contracted implicitly; the fused
// multiply-adds that are used are explicit fma() calls, the same ones in
// the host restatement, and only inside the predictor and the eigenvalue
// solvers, whose results the reference computes by other algorithms
// anyway.  What becomes a callback input whose Jacobian is then taken by
// forward differences (face states, time-step averages and gradients, B
// path points) and the FD quotients follow the reference build's own
// rounding: each product and sum rounded on its own, in the summation
// order of the Eigen kernel that evaluates it, quotients correctly rounded.  This matters more than
// usual here: the Rusanov and CFL eigenvalues come from a
// forward-difference Jacobian with step h = 2^-26 max(|q|, 1)
// (src/eigs/NumericalDiff.h:6-44), which turns any last-bit change of its
// input state into a ~1e-8 relative change of the Jacobian.
#pragma once

#ifndef __CUDACC_RTC__
#include <cstdint>
#endif

namespace pypde {

constexpr int MAXN = 8;
constexpr double SQRT_EPS = 1.4901161193847656e-08; // sqrt(2^-52) = 2^-26
constexpr double DBL_EPS = 2.220446049250313e-16;
constexpr double DBL_MAX_VAL = 1.7976931348623157e308;
constexpr unsigned long long INF_BITS = 0x7ff0000000000000ULL;

// |x| as its bit pattern: for x not NaN, a > b as doubles exactly when
// mag_bits(a) > mag_bits(b) as integers; zero is 0.
__host__ __device__ __forceinline__ unsigned long long mag_bits(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
#else
  unsigned long long u;
  __builtin_memcpy(&u, &x, 8);
  return u & 0x7fffffffffffffffULL;
#endif
}
constexpr double WENO_LAMS = 1.0;  // weno.h:8
constexpr double WENO_LAMC = 1e5;  // weno.h:9
constexpr double WENO_EPS = 1e-14; // weno.h:10
constexpr int DG_IT = 50;          // dg.h:8
constexpr double DG_TOL = 6e-6;    // dg.h:9

// Constant tables of one order N (src/poly/basis.cpp,
// src/solvers/weno/weno_matrices.cpp, src/solvers/dg/dg_matrices.cpp).
struct Tables {
  int N;
  double nodes[MAXN];
  double wghts[MAXN];
  double dervals[MAXN * MAXN]; // DERVALS[i*N+j] = psi_j'(x_i)
  double endvals[2 * MAXN];    // ENDVALS[e*N+j] = psi_j(e)
  double dgmat[MAXN * MAXN];
  double dgmat_inv[MAXN * MAXN];
  double weno_inv[4][MAXN * MAXN];
  double sig[MAXN * MAXN];
};

template <int B, int E> struct IPow {
  static constexpr int value = B * IPow<B, E - 1>::value;
};
template <int B> struct IPow<B, 0> {
  static constexpr int value = 1;
};

// ---------------------------------------------------------------------
// Eigenvalues of a general real V x V matrix: Householder reduction to
// Hessenberg form, then the Francis implicit double-shift QR iteration
// with Wilkinson's deflation test (Golub & Van Loan, Matrix Computations,
// Alg. 7.4.2 and 7.5.1).  Replaces Eigen::EigenSolver / Spectra
// (src/eigs/system.cpp:28-43).  Same operation order as the host
// restatement.  Returns max |lambda|, NaN if the iteration fails.
// ---------------------------------------------------------------------
template <int V>
__device__ __forceinline__ void hessenberg_inplace(double *a) {
#define A_(i, j) a[(i) * V + (j)]
  for (int k = 0; k < V - 2; k++) {
    double v[V];
    double alpha = 0, scale = 0;
    for (int i = k + 1; i < V; i++)
      scale += fabs(A_(i, k));
    if (scale == 0.0)
      continue;
    for (int i = k + 1; i < V; i++) {
      v[i] = A_(i, k) / scale;
      alpha += v[i] * v[i];
    }
    double g = sqrt(alpha);
    if (v[k + 1] > 0)
      g = -g;
    double h = alpha - v[k + 1] * g;
    v[k + 1] -= g;
    for (int j = k; j < V; j++) {
      double s = 0;
      for (int i = k + 1; i < V; i++)
        s += v[i] * A_(i, j);
      s /= h;
      for (int i = k + 1; i < V; i++)
        A_(i, j) -= s * v[i];
    }
    for (int i = 0; i < V; i++) {
      double s = 0;
      for (int j = k + 1; j < V; j++)
        s += A_(i, j) * v[j];
      s /= h;
      for (int j = k + 1; j < V; j++)
        A_(i, j) -= s * v[j];
    }
    A_(k + 1, k) = g * scale;
    for (int i = k + 2; i < V; i++)
      A_(i, k) = 0.0;
  }
}

template <int V>
__device__ __noinline__ double max_abs_eig_qr(double *a) {
  if (V == 1)
    return fabs(a[0]);
  hessenberg_inplace<V>(a);
  double wr[V], wi[V];
  double norm = 0;
  for (int i = 0; i < V; i++)
    for (int j = (i > 0 ? i - 1 : 0); j < V; j++)
      norm += fabs(A_(i, j));
  int hi = V - 1, its = 0, total = 0;
  double exshift = 0.0;
  while (hi >= 0) {
    int l;
    for (l = hi; l > 0; l--) {
      double s = fabs(A_(l - 1, l - 1)) + fabs(A_(l, l));
      if (s == 0.0)
        s = norm;
      if (fabs(A_(l, l - 1)) <= DBL_EPS * s) {
        A_(l, l - 1) = 0.0;
        break;
      }
    }
    if (l == hi) {
      wr[hi] = A_(hi, hi) + exshift;
      wi[hi] = 0.0;
      hi--;
      its = 0;
      continue;
    }
    if (l == hi - 1) {
      double p = 0.5 * (A_(hi - 1, hi - 1) - A_(hi, hi));
      double qq = p * p + A_(hi, hi - 1) * A_(hi - 1, hi);
      double zz = sqrt(fabs(qq));
      double x = A_(hi, hi) + exshift;
      if (qq >= 0.0) {
        zz = (p >= 0) ? p + zz : p - zz;
        wr[hi - 1] = x + zz;
        wr[hi] = (zz != 0.0) ? x - A_(hi, hi - 1) * A_(hi - 1, hi) / zz
                             : x + zz;
        wi[hi - 1] = wi[hi] = 0.0;
      } else {
        wr[hi - 1] = wr[hi] = x + p;
        wi[hi - 1] = zz;
        wi[hi] = -zz;
      }
      hi -= 2;
      its = 0;
      continue;
    }
    double x = A_(hi, hi), y = A_(hi - 1, hi - 1);
    double w = A_(hi, hi - 1) * A_(hi - 1, hi);
    if (its == 10 || its == 20) {
      exshift += x;
      for (int i = 0; i <= hi; i++)
        A_(i, i) -= x;
      double s = fabs(A_(hi, hi - 1)) + fabs(A_(hi - 1, hi - 2));
      x = y = 0.75 * s;
      w = -0.4375 * s * s;
    }
    its++;
    if (++total > 40 * V)
      return __longlong_as_double(0x7ff8000000000000ULL);
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
    for (int k = m; k <= hi - 1; k++) {
      bool notlast = (k != hi - 1);
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
      for (int j = k; j <= hi; j++) {
        double pp = A_(k, j) + q * A_(k + 1, j);
        if (notlast) {
          pp += r * A_(k + 2, j);
          A_(k + 2, j) -= pp * zz;
        }
        A_(k + 1, j) -= pp * y;
        A_(k, j) -= pp * x;
      }
      int ihi = (hi < k + 3) ? hi : k + 3;
      for (int i = l; i <= ihi; i++) {
        double pp = x * A_(i, k) + y * A_(i, k + 1);
        if (notlast) {
          pp += zz * A_(i, k + 2);
          A_(i, k + 2) -= pp * r;
        }
        A_(i, k + 1) -= pp * q;
        A_(i, k) -= pp;
      }
    }
  }
  double mx = 0;
  for (int i = 0; i < V; i++) {
    double rr = (wi[i] == 0.0) ? fabs(wr[i])
                               : sqrt(wr[i] * wr[i] + wi[i] * wi[i]);
    if (rr > mx)
      mx = rr;
  }
  return mx;
#undef A_
}

// ---------------------------------------------------------------------
// FP32 eigenvalues (Householder + Francis, same algorithm in float): the
// shifts of the FP64 refinement.  FP32 runs on this part at ~70x the FP64
// rate, so the QR sweeps cost next to nothing; only the refinement below
// uses the FP64 pipe.  Returns 0, or -1 if the iteration fails.
// ---------------------------------------------------------------------
template <int V>
__device__ __noinline__ int eig_vals_f(float *a, float *wr, float *wi) {
#define AF(i, j) a[(i) * V + (j)]
  for (int k = 0; k < V - 2; k++) {
    float v[V];
    float alpha = 0, scale = 0;
    for (int i = k + 1; i < V; i++)
      scale += fabsf(AF(i, k));
    if (scale == 0.0f)
      continue;
    for (int i = k + 1; i < V; i++) {
      v[i] = AF(i, k) / scale;
      alpha += v[i] * v[i];
    }
    float g = sqrtf(alpha);
    if (v[k + 1] > 0)
      g = -g;
    float h = alpha - v[k + 1] * g;
    v[k + 1] -= g;
    for (int j = k; j < V; j++) {
      float s = 0;
      for (int i = k + 1; i < V; i++)
        s += v[i] * AF(i, j);
      s /= h;
      for (int i = k + 1; i < V; i++)
        AF(i, j) -= s * v[i];
    }
    for (int i = 0; i < V; i++) {
      float s = 0;
      for (int j = k + 1; j < V; j++)
        s += AF(i, j) * v[j];
      s /= h;
      for (int j = k + 1; j < V; j++)
        AF(i, j) -= s * v[j];
    }
    AF(k + 1, k) = g * scale;
    for (int i = k + 2; i < V; i++)
      AF(i, k) = 0.0f;
  }
  const float eps = 1.1920929e-07f;
  float norm = 0;
  for (int i = 0; i < V; i++)
    for (int j = (i > 0 ? i - 1 : 0); j < V; j++)
      norm += fabsf(AF(i, j));
  int hi = V - 1, its = 0, total = 0;
  float exshift = 0.0f;
  while (hi >= 0) {
    int l;
    for (l = hi; l > 0; l--) {
      float s = fabsf(AF(l - 1, l - 1)) + fabsf(AF(l, l));
      if (s == 0.0f)
        s = norm;
      if (fabsf(AF(l, l - 1)) <= eps * s) {
        AF(l, l - 1) = 0.0f;
        break;
      }
    }
    if (l == hi) {
      wr[hi] = AF(hi, hi) + exshift;
      wi[hi] = 0.0f;
      hi--;
      its = 0;
      continue;
    }
    if (l == hi - 1) {
      float p = 0.5f * (AF(hi - 1, hi - 1) - AF(hi, hi));
      float qq = p * p + AF(hi, hi - 1) * AF(hi - 1, hi);
      float zz = sqrtf(fabsf(qq));
      float x = AF(hi, hi) + exshift;
      if (qq >= 0.0f) {
        zz = (p >= 0) ? p + zz : p - zz;
        wr[hi - 1] = x + zz;
        wr[hi] = (zz != 0.0f) ? x - AF(hi, hi - 1) * AF(hi - 1, hi) / zz
                              : x + zz;
        wi[hi - 1] = wi[hi] = 0.0f;
      } else {
        wr[hi - 1] = wr[hi] = x + p;
        wi[hi - 1] = zz;
        wi[hi] = -zz;
      }
      hi -= 2;
      its = 0;
      continue;
    }
    float x = AF(hi, hi), y = AF(hi - 1, hi - 1);
    float w = AF(hi, hi - 1) * AF(hi - 1, hi);
    if (its == 10 || its == 20) {
      exshift += x;
      for (int i = 0; i <= hi; i++)
        AF(i, i) -= x;
      float s = fabsf(AF(hi, hi - 1)) + fabsf(AF(hi - 1, hi - 2));
      x = y = 0.75f * s;
      w = -0.4375f * s * s;
    }
    its++;
    if (++total > 40 * V)
      return -1;
    int m;
    float p = 0, q = 0, r = 0;
    for (m = hi - 2; m >= l; m--) {
      float zz = AF(m, m);
      float rr = x - zz, ss = y - zz;
      p = (rr * ss - w) / AF(m + 1, m) + AF(m, m + 1);
      q = AF(m + 1, m + 1) - zz - rr - ss;
      r = AF(m + 2, m + 1);
      float s = fabsf(p) + fabsf(q) + fabsf(r);
      p /= s;
      q /= s;
      r /= s;
      if (m == l)
        break;
      float u = fabsf(AF(m, m - 1)) * (fabsf(q) + fabsf(r));
      float vv = fabsf(p) * (fabsf(AF(m - 1, m - 1)) + fabsf(zz) +
                             fabsf(AF(m + 1, m + 1)));
      if (u <= eps * vv)
        break;
    }
    for (int i = m + 2; i <= hi; i++) {
      AF(i, i - 2) = 0.0f;
      if (i > m + 2)
        AF(i, i - 3) = 0.0f;
    }
    for (int k = m; k <= hi - 1; k++) {
      bool notlast = (k != hi - 1);
      if (k != m) {
        p = AF(k, k - 1);
        q = AF(k + 1, k - 1);
        r = notlast ? AF(k + 2, k - 1) : 0.0f;
        x = fabsf(p) + fabsf(q) + fabsf(r);
        if (x == 0.0f)
          continue;
        p /= x;
        q /= x;
        r /= x;
      }
      float s = sqrtf(p * p + q * q + r * r);
      if (p < 0)
        s = -s;
      if (k != m)
        AF(k, k - 1) = -s * x;
      else if (l != m)
        AF(k, k - 1) = -AF(k, k - 1);
      p += s;
      x = p / s;
      y = q / s;
      float zz = r / s;
      q /= p;
      r /= p;
      for (int j = k; j <= hi; j++) {
        float pp = AF(k, j) + q * AF(k + 1, j);
        if (notlast) {
          pp += r * AF(k + 2, j);
          AF(k + 2, j) -= pp * zz;
        }
        AF(k + 1, j) -= pp * y;
        AF(k, j) -= pp * x;
      }
      int ihi = (hi < k + 3) ? hi : k + 3;
      for (int i = l; i <= ihi; i++) {
        float pp = x * AF(i, k) + y * AF(i, k + 1);
        if (notlast) {
          pp += zz * AF(i, k + 2);
          AF(i, k + 2) -= pp * r;
        }
        AF(i, k + 1) -= pp * q;
        AF(i, k) -= pp;
      }
    }
  }
  return 0;
#undef AF
}

// FP32 LU with partial pivoting (whole-row swaps) of the V x V matrix A in
// place; ud gets the reciprocals of the pivots.  -1 on a zero pivot.
template <int V>
__device__ __forceinline__ int lu32(float *A, int *piv, float *ud) {
  for (int k = 0; k < V; k++) {
    int p = k;
    for (int i = k + 1; i < V; i++)
      if (fabsf(A[i * V + k]) > fabsf(A[p * V + k]))
        p = i;
    piv[k] = p;
    if (A[p * V + k] == 0.0f)
      return -1;
    if (p != k)
      for (int j = 0; j < V; j++) {
        float t = A[k * V + j];
        A[k * V + j] = A[p * V + j];
        A[p * V + j] = t;
      }
    ud[k] = 1.0f / A[k * V + k];
    for (int i = k + 1; i < V; i++) {
      float f = A[i * V + k] * ud[k];
      A[i * V + k] = f;
      for (int j = k + 1; j < V; j++)
        A[i * V + j] = fmaf(-f, A[k * V + j], A[i * V + j]);
    }
  }
  return 0;
}

// x <- A^{-1} x with the factors of lu32 (permute, unit L, then U).
template <int V>
__device__ __forceinline__ void lu32_solve(const float *A, const int *piv,
                                           const float *ud, float *x) {
  for (int k = 0; k < V; k++)
    if (piv[k] != k) {
      float t = x[k];
      x[k] = x[piv[k]];
      x[piv[k]] = t;
    }
  for (int k = 0; k < V; k++)
    for (int i = k + 1; i < V; i++)
      x[i] = fmaf(-A[i * V + k], x[k], x[i]);
  for (int i = V - 1; i >= 0; i--) {
    float sacc = x[i];
    for (int j = i + 1; j < V; j++)
      sacc = fmaf(-A[i * V + j], x[j], sacc);
    x[i] = sacc * ud[i];
  }
}

// One real eigenvalue refined from the FP32 shift lam0 (an eigenvalue of M
// rounded to FP32) by the iterative refinement of an eigenpair of Dongarra,
// Moler and Wilkinson (SIAM J. Numer. Anal. 20, 1983):
//   FP32: x from two inverse-iteration steps with the LU of Mf - lam0 I
//         (Mf = M rounded to FP32), scaled so that x_s = 1 at its largest
//         entry s; the LU of B = Mf - lam0 I with column s replaced by -x.
//   FP64 residual, FP32 correction, three times:
//         r = lam x - M x;  z = B^{-1} r;  lam += z_s;  x_j += z_j (j != s)
// Converges linearly at a rate of about eps_32 cond(B).  Returns -1 on a
// zero FP32 pivot, a vector that vanishes or is not finite, or a last
// correction larger than 1e-10 |lam|.  Same operations and order as the
// host restatement's refine_real.
template <int V>
__device__ __forceinline__ int refine_real(const double *M, double lam0d,
                                           double *lam) {
  float A[V * V], ud[V], x[V], z[V];
  int piv[V];
  const float lam0 = (float)lam0d;
#pragma unroll
  for (int i = 0; i < V * V; i++)
    A[i] = (float)M[i];
#pragma unroll
  for (int i = 0; i < V; i++)
    A[i * V + i] = A[i * V + i] - lam0;
  if (lu32<V>(A, piv, ud) != 0)
    return -1;
#pragma unroll
  for (int i = 0; i < V; i++)
    x[i] = 1.0f;
  int s = 0;
  for (int it = 0; it < 2; it++) {
    lu32_solve<V>(A, piv, ud, x);
    float mx = 0.0f;
    s = 0;
    for (int i = 0; i < V; i++)
      if (fabsf(x[i]) > mx) {
        mx = fabsf(x[i]);
        s = i;
      }
    if (!(mx > 0.0f) || !(mx <= 3.0e38f))
      return -1;
    const float ix = 1.0f / x[s];
    for (int i = 0; i < V; i++)
      x[i] *= ix;
  }
  x[s] = 1.0f;
#pragma unroll
  for (int i = 0; i < V * V; i++)
    A[i] = (float)M[i];
  for (int i = 0; i < V; i++) {
    A[i * V + i] = A[i * V + i] - lam0;
    A[i * V + s] = -x[i];
  }
  if (lu32<V>(A, piv, ud) != 0)
    return -1;
  double xd[V], l = (double)lam0, dl = 0;
#pragma unroll
  for (int i = 0; i < V; i++)
    xd[i] = (double)x[i];
  for (int it = 0; it < 3; it++) {
    for (int i = 0; i < V; i++) {
      double acc = 0;
#pragma unroll
      for (int j = 0; j < V; j++)
        acc = fma(M[i * V + j], xd[j], acc);
      z[i] = (float)fma(l, xd[i], -acc);
    }
    lu32_solve<V>(A, piv, ud, z);
    dl = (double)z[s];
    l += dl;
    for (int i = 0; i < V; i++)
      if (i != s)
        xd[i] += (double)z[i];
  }
  if (!(fabs(dl) <= 1e-10 * fabs(l)))
    return -1;
  *lam = l;
  return 0;
}

// max |eigenvalue| (a4): FP32 eigenvalues choose the candidates of largest
// modulus (within 2^-10 of the largest); each is refined in FP64.  Complex
// or nearly coincident candidates, a failed FP32 iteration, a singular
// shift, or a refinement that moves its shift by more than 1e-5 relative
// fall back to the FP64 Francis QR.  Same algorithm and operation order as
// the host restatement, so both give the same bits.
template <int V>
__device__ __noinline__ double max_abs_eig(double *a) {
  if (V == 1)
    return fabs(a[0]);
  float af[V * V], wr[V], wi[V];
#pragma unroll
  for (int i = 0; i < V * V; i++)
    af[i] = (float)a[i];
  if (eig_vals_f<V>(af, wr, wi) != 0)
    return max_abs_eig_qr<V>(a);
  float mf = 0;
  for (int i = 0; i < V; i++) {
    float m = (wi[i] == 0.0f) ? fabsf(wr[i])
                              : sqrtf(wr[i] * wr[i] + wi[i] * wi[i]);
    if (m > mf)
      mf = m;
  }
  if (!(mf > 0.0f) || mf != mf || mf > 3.0e38f)
    return max_abs_eig_qr<V>(a);
  float thr = mf - mf * 0.0009765625f;
  int cand[V], nc = 0;
  for (int i = 0; i < V; i++) {
    float m = (wi[i] == 0.0f) ? fabsf(wr[i])
                              : sqrtf(wr[i] * wr[i] + wi[i] * wi[i]);
    if (m >= thr) {
      if (wi[i] != 0.0f)
        return max_abs_eig_qr<V>(a);
      cand[nc++] = i;
    }
  }
  for (int i = 0; i < nc; i++)
    for (int j = i + 1; j < nc; j++)
      if (fabsf(wr[cand[i]] - wr[cand[j]]) <= 1e-4f * mf)
        return max_abs_eig_qr<V>(a);
  double best = 0;
  for (int i = 0; i < nc; i++) {
    double lam;
    double lam0 = (double)wr[cand[i]];
    if (refine_real<V>(a, lam0, &lam) != 0)
      return max_abs_eig_qr<V>(a);
    if (!(fabs(lam - lam0) <= 1e-5 * fabs(lam0)))
      return max_abs_eig_qr<V>(a);
    best = fmax(best, fabs(lam));
  }
  return best;
}

// The reciprocal of an FD step h split in two, y_hi + y_lo = 1/h to about
// 2^-106 relative: y_hi = RN(1/h) (one division per column), and y_lo from
// the residual 1 - h y_hi, which an FMA gives exactly.  ok: h is far
// enough from the top of the exponent range that y_lo is not subnormal.
struct FdStep {
  double h, hi, lo;
  bool ok;
};
__device__ __forceinline__ FdStep fd_step(double h) {
  FdStep s;
  s.h = h;
  s.hi = 1.0 / h;
  s.lo = fma(-h, s.hi, 1.0) * s.hi;
  s.ok = h <= 0x1p+900;
  return s;
}

// The rare quotients fd_div does not form itself, out of line.
static __device__ __noinline__ double fd_div_slow(double x, double h) {
  return x / h;
}

// x / h correctly rounded, as NumericalDiff.h:31 divides each entry,
// without a division per entry: q0 = x y_hi + x y_lo is within half an ulp
// and a hair of x / h, so it is a faithful quotient and its remainder
// x - h q0 is exact (one FMA); one correction q0 + (x - h q0) y_hi then
// rounds to the correctly rounded quotient, by Markstein's theorem (P.
// Markstein, IBM J. Res. Dev. 34 (1990) 111-119; Cornea, Golliver and
// Markstein, ARITH 14 (1999), Theorem 1: y_hi within half an ulp of 1/h,
// q0 within one ulp of x / h).  A zero x gives the signed zero x y_hi (the
// quotient's bits); a quotient beyond 2^+-900, where a remainder could be
// subnormal, and non-finite values take the division itself.  The tests
// are on the integer pipe.
__device__ __forceinline__ double fd_div(double x, const FdStep &s) {
  const unsigned long long xb = (unsigned long long)__double_as_longlong(x);
  if ((xb << 1) == 0ULL)
    return x * s.hi;
  const double q0 = fma(x, s.hi, x * s.lo);
  const unsigned e =
      (unsigned)(((unsigned long long)__double_as_longlong(q0) >> 52) & 0x7ffu);
  if (e - 123u > 1800u || !s.ok)
    return fd_div_slow(x, s.h);
  return fma(fma(-q0, s.h, x), s.hi, q0);
}

// Forward-difference Jacobian of F (NumericalDiff.h:6-44 with its default
// forwardMode=true, which both call sites use: system.cpp:15, :58), each
// entry (v2 - v1) / h correctly rounded as NumericalDiff.h:31 divides it:
// the Jacobian equals the reference's bit for bit on the same state (the
// one-ulp differences of a reciprocal multiply, small as they are, move
// every step's dt and add up over a long run).
// wrt_dq: perturb dq[d*V+i] (second-order form) instead of q[i].
template <class Sys>
__device__ __forceinline__ void fd_jacobian(double *jac, double *q, double *dq,
                                            int d, bool wrt_dq,
                                            double *f0 = nullptr) {
  constexpr int V = Sys::V;
  double v1[V], v2[V];
  Sys::F(v1, q, dq, d);
  if (f0) // F(q) itself, reused by the Rusanov flux
    for (int r = 0; r < V; r++)
      f0[r] = v1[r];
  for (int i = 0; i < V; i++) {
    double *qi = wrt_dq ? dq + d * V + i : q + i;
    double qi0 = *qi;
    double h = fmax(SQRT_EPS * fabs(qi0), SQRT_EPS);
    *qi += h;
    Sys::F(v2, q, dq, d);
    *qi = qi0;
    const FdStep fs = fd_step(h);
    for (int r = 0; r < V; r++)
      jac[r * V + i] = fd_div(v2[r] - v1[r], fs);
  }
}

// A system that declares EIG_ACTIVE and eig_active(d, k) names, for each
// direction d, the EIG_ACTIVE variables that its flux in direction d
// transports (k = 0 .. EIG_ACTIVE-1, ascending); the others are passive:
// no flux component depends on them and their own flux is constant.
template <class...> using void_t_ = void;
template <class S, class = void> struct HasEigActive {
  static constexpr bool value = false;
};
template <class S>
struct HasEigActive<S, void_t_<decltype(S::EIG_ACTIVE)>> {
  static constexpr bool value = true;
};

// max |eigenvalue| of the system matrix M in direction d (destroyed).
// Where the system declares its passive variables and their rows and
// columns of M are zero off the diagonal (checked), each carries the
// eigenvalue M_ii, and the rest of the spectrum is that of the active
// block (the permutation step of Parlett and Reinsch's balancing, Numer.
// Math. 13, 1969, with the permutation known in advance): max|eig| is
// taken over the active block and the passive diagonal.  The block has the
// same size for every matrix of the system, so all threads run the same
// solver.  Otherwise, or if a passive diagonal entry is not finite, the
// full matrix.  Same steps as the host restatement.
template <class Sys>
__device__ __forceinline__ double max_abs_eig_sys(double *M, int d) {
  constexpr int V = Sys::V;
  if constexpr (HasEigActive<Sys>::value) {
    constexpr int MA = Sys::EIG_ACTIVE;
    static_assert(MA >= 1 && MA < V, "EIG_ACTIVE out of range");
    unsigned active = 0;
#pragma unroll
    for (int k = 0; k < MA; k++)
      active |= 1u << Sys::eig_active(d, k);
    bool ok = true;
    double iso = 0.0;
#pragma unroll
    for (int i = 0; i < V; i++) {
      if (active >> i & 1u)
        continue;
#pragma unroll
      for (int j = 0; j < V; j++)
        if (j != i && (M[i * V + j] != 0.0 || M[j * V + i] != 0.0))
          ok = false;
      const double di = fabs(M[i * V + i]);
      if (!(di <= DBL_MAX_VAL))
        ok = false;
      else if (di > iso)
        iso = di;
    }
    if (ok) {
      double S[MA * MA];
#pragma unroll
      for (int r = 0; r < MA; r++)
#pragma unroll
        for (int c = 0; c < MA; c++)
          S[r * MA + c] = M[Sys::eig_active(d, r) * V + Sys::eig_active(d, c)];
      const double r = max_abs_eig<MA>(S);
      return (r < iso) ? iso : r;
    }
  }
  return max_abs_eig<V>(M);
}

// The FD Jacobian of F restricted to the active block, for a system that
// declares its passive variables (no B): only the active columns are
// evaluated (no flux component depends on a passive variable), each entry
// exactly as fd_jacobian computes it, into the EIG_ACTIVE x EIG_ACTIVE
// block S.  The passive rows of those columns must come out zero (their
// flux is constant); returns false if one does not.
template <class Sys>
__device__ __forceinline__ bool fd_jacobian_active(double *S, double *q,
                                                   double *dq, int d,
                                                   double *f0) {
  constexpr int V = Sys::V, MA = Sys::EIG_ACTIVE;
  unsigned active = 0;
#pragma unroll
  for (int k = 0; k < MA; k++)
    active |= 1u << Sys::eig_active(d, k);
  double v1[V], v2[V];
  Sys::F(v1, q, dq, d);
  if (f0)
#pragma unroll
    for (int r = 0; r < V; r++)
      f0[r] = v1[r];
  bool ok = true;
  for (int k = 0; k < MA; k++) {
    const int i = Sys::eig_active(d, k);
    const double qi0 = q[i];
    const double h = fmax(SQRT_EPS * fabs(qi0), SQRT_EPS);
    q[i] += h;
    Sys::F(v2, q, dq, d);
    q[i] = qi0;
    const FdStep fs = fd_step(h);
    int rk = 0;
#pragma unroll
    for (int r = 0; r < V; r++) {
      // a passive entry is zero exactly when v2 - v1 is: only the active
      // entries are divided
      if (active >> r & 1u)
        S[(rk++) * MA + k] = fd_div(v2[r] - v1[r], fs);
      else if (v2[r] - v1[r] != 0.0)
        ok = false;
    }
  }
  return ok;
}

// system_matrix + max|eig| (src/eigs/system.cpp:6-51).  For a system with
// passive variables and no B, the Jacobian is built on the active block
// directly; its passive eigenvalues are zero (constant flux).  If a
// passive row is not zero, the full matrix path below decides.
template <class Sys>
__device__ __forceinline__ double max_abs_eigs(double *q, double *dq, int d,
                                               double *f0 = nullptr) {
  constexpr int V = Sys::V;
  if constexpr (HasEigActive<Sys>::value && Sys::HAS_F && !Sys::HAS_B) {
    constexpr int MA = Sys::EIG_ACTIVE;
    double S[MA * MA];
    if (fd_jacobian_active<Sys>(S, q, dq, d, f0))
      return max_abs_eig<MA>(S);
  }
  double M[V * V];
  if (Sys::HAS_F)
    fd_jacobian<Sys>(M, q, dq, d, false, f0);
  else
    for (int i = 0; i < V * V; i++)
      M[i] = 0.0;
  if (Sys::HAS_B) {
    double b[V * V];
    Sys::B(b, q, d);
    for (int i = 0; i < V * V; i++)
      M[i] += b[i];
  }
  return max_abs_eig_sys<Sys>(M, d);
}

// max_abs_eigs as a call rather than inlined: the face kernel evaluates it
// twice per face point (both states), and one out-of-line copy lets the two
// evaluations share their registers and stack instead of spilling.
template <class Sys>
__device__ __noinline__ double max_abs_eigs_call(double *q, double *dq, int d,
                                                 double *f0) {
  return max_abs_eigs<Sys>(q, dq, d, f0);
}

// The FD Jacobian + B itself (src/eigs/system.cpp:6-26).
template <class Sys>
__device__ __forceinline__ void system_matrix(double *M, double *q, double *dq,
                                              int d) {
  constexpr int V = Sys::V;
  if (Sys::HAS_F)
    fd_jacobian<Sys>(M, q, dq, d, false);
  else
    for (int i = 0; i < V * V; i++)
      M[i] = 0.0;
  if (Sys::HAS_B) {
    double b[V * V];
    Sys::B(b, q, d);
    for (int i = 0; i < V * V; i++)
      M[i] += b[i];
  }
}

// 2 (N+1) / dX_d * max|eig(dF/d(dq_d))| (src/eigs/system.cpp:53-61)
template <class Sys>
__device__ __forceinline__ double max_abs_eigs_2nd(double *q, double *dq, int d,
                                                   int N, double dXd) {
  constexpr int V = Sys::V;
  double M[V * V];
  fd_jacobian<Sys>(M, q, dq, d, true);
  return 2 * (N + 1) / dXd * max_abs_eig<V>(M);
}

// One output lane of the column-major matrix-vector product that the
// reference's Eigen 3.3 build evaluates for `row * matrix` and
// `vector^T * matrix` (its GeneralMatrixVector.h:88-315, SSE2 packets of
// two doubles, result buffer 16-byte aligned): sum_k a[k] x[k xstride]
// over n columns.  Columns go in blocks of four from column `rot` on; a
// packet lane adds each block as ((c0 + c1) + (c2 + c3)), the odd last
// lane left to right; leftover columns follow left to right, and with
// rot = 1 column 0 comes last.  Each product and sum is rounded on its
// own, as the reference's x86-64 build (no FMA) rounds them.  Used where
// the result is a callback input whose flux Jacobian is then taken by
// forward differences (step ~1e-8 relative), which amplifies a last-bit
// change of it ~1e8-fold: the quadrature averages of the time step
// (stepper.cpp:49,53) and the face states (evaluations.cpp:49-70).
__device__ __forceinline__ double gemv_lane(const double *a, const double *x,
                                            int xstride, int n, bool packet,
                                            bool rot) {
  double s = 0;
  const int k0 = rot ? 1 : 0;
  const int bound = ((n - k0) / 4) * 4 + k0;
  for (int k = k0; k < bound; k += 4) {
    double a0 = a[k] * x[k * xstride], a1 = a[k + 1] * x[(k + 1) * xstride];
    double a2 = a[k + 2] * x[(k + 2) * xstride];
    double a3 = a[k + 3] * x[(k + 3) * xstride];
    if (packet)
      s = s + ((a0 + a1) + (a2 + a3));
    else
      s = (((s + a0) + a1) + a2) + a3;
  }
  for (int k = bound; k < n; k++)
    s = s + a[k] * x[k * xstride];
  if (rot)
    s = s + a[0] * x[0];
  return s;
}

// Whether that product skips its first column: Eigen does so, to load the
// later columns aligned, when there are V > 1 result lanes, the column
// stride (in doubles) is odd and the first element lies an odd number of
// doubles past a 16-byte boundary (the reference's buffers start on one).
__device__ __forceinline__ bool gemv_rot(int V, long long stride,
                                         long long offset) {
  return V > 1 && (stride & 1) && (offset & 1);
}

// The FD step of the stiff predictor's source Jacobian: the power of two
// h = 2^(max(floor(log2 |x|), 0) - 26), within a factor two below
// sqrt(eps) max(|x|, 1), so that 1/h is exact and the difference
// quotients are multiplications.  Zero, subnormal, infinite and NaN x take
// h = 2^-26.  The matrix only steers the simplified Newton iteration; the
// residual that it drives to the tolerance is evaluated exactly.
__device__ __forceinline__ void fd_step_pow2(double x, double &h, double &ih) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  int E = (e == 0 || e == 0x7ff) ? 0 : e - 1023;
  if (E < 0)
    E = 0;
  h = __longlong_as_double((long long)((unsigned long long)(E - 26 + 1023) << 52));
  ih = __longlong_as_double((long long)((unsigned long long)(26 - E + 1023) << 52));
}

// Non-negative doubles order like their bit patterns: max via integer
// atomics.  NaN is skipped, as std::max(MAX, NaN) keeps MAX
// (stepper.cpp:65).
__device__ __forceinline__ void atomic_max_pos(double *addr, double v) {
  if (!(v == v))
    return;
  atomicMax(reinterpret_cast<unsigned long long *>(addr),
            static_cast<unsigned long long>(__double_as_longlong(v)));
}

} // namespace pypde
