// systems.cuh -- built-in device callback systems (the user's F/B/S of
// pypde's pde_solver, src/api.h:4-10, compiled ahead of time).
//
// A system is a struct with
//   static constexpr int V, NDIM; HAS_F, HAS_B, HAS_S, SECOND_ORDER flags
//   F(out[V], Q[V], dQ[NDIM*V], d)   flux in direction d
//   B(out[V*V] row-major, Q[V], d)   non-conservative matrix
//   S(out[V], Q[V])                  source
// exactly the reference callback signatures (pypde/cfuncs.py:6-8).  User
// systems compiled at run time (NVRTC) provide the same struct.
//
// Formulas and operation order match the host test callbacks, so host and
// device produce the same bits (the kernels are compiled without implicit
// FMA contraction, and the callbacks use no fma()):
//   Euler<D>     V = D+2   (rho, m_0..m_{D-1}, E), gamma = 1.4
//   Cattaneo<D>  V = 2D+3  Euler + relaxing heat flux q + passive
//                s = log10(tau); T = p/rho; F_d adds q_d to the energy flux
//                and kappa_h T to q_d (kappa_h = kappa/tau_ref = 1); the
//                local tau (1/tau = 10^-s) enters only S_q = -q/tau
//   Ncp<D>       V = 3, F, B and S (a non-conservative test system)
//   Burgers2     V = 1, D = 1, second-order form F(Q, dQ, d)
#pragma once

namespace pypde {

// 10^x = 2^n e^r with n = round(x log2 10), |r| <= ln2/2, and e^r by its
// Taylor polynomial of degree 16 in Horner form (truncation below 1e-22),
// from IEEE +, *, floor and ldexp only, so that host and device agree
// bitwise.  The coefficients are the doubles nearest to 1/k!.  T = float
// gives the same recipe in FP32 (for the FP32 Newton sweeps).
template <class T> __device__ __forceinline__ T pow10_portable(T x) {
  constexpr double c[17] = {
      1.0, 1.0, 0.5, 0.16666666666666666,
      0.041666666666666664, 0.008333333333333333, 0.001388888888888889, 0.0001984126984126984,
      2.48015873015873e-05, 2.7557319223985893e-06, 2.755731922398589e-07, 2.505210838544172e-08,
      2.08767569878681e-09, 1.6059043836821613e-10, 1.1470745597729725e-11, 7.647163731819816e-13,
      4.779477332387385e-14};
  T y = x * T(3.321928094887362);
  T n = floor(y + T(0.5));
  T r = (y - n) * T(0.6931471805599453);
  T p = T(c[16]);
#pragma unroll
  for (int k = 15; k >= 0; k--)
    p = p * r + T(c[k]);
  return ldexp(p, (int)n);
}

// The callbacks are templates on the scalar type: double for every form,
// float for the FP32 Newton sweeps of the mixed-precision form (HAS_FP32).
template <int D> struct EulerCore {
  template <class T>
  static __device__ __forceinline__ T flux(T *out, const T *Q, int d) {
    T r = Q[0];
    T ke = T(0.0);
#pragma unroll
    for (int i = 0; i < D; i++)
      ke += Q[1 + i] * Q[1 + i];
    T p = (T(1.4) - T(1.0)) * (Q[D + 1] - T(0.5) * ke / r);
    T ud = Q[1 + d] / r;
    out[0] = Q[1 + d];
#pragma unroll
    for (int i = 0; i < D; i++)
      out[1 + i] = Q[1 + i] * ud;
    out[1 + d] += p;
    out[D + 1] = (Q[D + 1] + p) * ud;
    return p;
  }
};

template <int D> struct Euler {
  static constexpr int V = D + 2, NDIM = D;
  static constexpr bool HAS_F = true, HAS_B = false, HAS_S = false;
  static constexpr bool SECOND_ORDER = false, HAS_FP32 = true;
  template <class T>
  static __device__ __forceinline__ void F(T *out, const T *Q, const T *, int d) {
    EulerCore<D>::flux(out, Q, d);
  }
  template <class T> static __device__ __forceinline__ void B(T *, const T *, int) {}
  template <class T> static __device__ __forceinline__ void S(T *, const T *) {}
};

template <int D> struct Cattaneo {
  static constexpr int V = 2 * D + 3, NDIM = D;
  // the flux in direction d transports rho, the momenta, E and q_d; the
  // other heat-flux components and log tau are passive
  static constexpr int EIG_ACTIVE = D + 3;
  static __host__ __device__ constexpr int eig_active(int d, int k) {
    return k < D + 2 ? k : D + 2 + d;
  }
  static constexpr bool HAS_F = true, HAS_B = false, HAS_S = true;
  static constexpr bool SECOND_ORDER = false, HAS_FP32 = true;
  template <class T>
  static __device__ __forceinline__ void F(T *out, const T *Q, const T *, int d) {
    T p = EulerCore<D>::flux(out, Q, d);
    T Tt = p / Q[0];
    out[D + 1] += Q[D + 2 + d];
#pragma unroll
    for (int i = 0; i < D; i++)
      out[D + 2 + i] = T(0.0);
    out[D + 2 + d] = T(1.0) * Tt;
    out[2 * D + 2] = T(0.0);
  }
  template <class T> static __device__ __forceinline__ void B(T *, const T *, int) {}
  template <class T>
  static __device__ __forceinline__ void S(T *out, const T *Q) {
    T inv_tau = pow10_portable<T>(-Q[2 * D + 2]);
#pragma unroll
    for (int i = 0; i < D + 2; i++)
      out[i] = T(0.0);
#pragma unroll
    for (int i = 0; i < D; i++)
      out[D + 2 + i] = -Q[D + 2 + i] * inv_tau;
    out[2 * D + 2] = T(0.0);
  }
};

template <class T> __device__ __forceinline__ T ncp_a(int d) {
  return d == 0 ? T(1.0) : (d == 1 ? T(0.5) : T(0.25));
}

template <int D> struct Ncp {
  static constexpr int V = 3, NDIM = D;
  static constexpr bool HAS_F = true, HAS_B = true, HAS_S = true;
  static constexpr bool SECOND_ORDER = false, HAS_FP32 = true;
  template <class T>
  static __device__ __forceinline__ void F(T *out, const T *Q, const T *, int d) {
    T a = ncp_a<T>(d);
    out[0] = a * (T(0.5) * Q[0] * Q[0]);
    out[1] = a * (Q[0] * Q[1]);
    out[2] = a * (Q[0] * Q[2]);
  }
  template <class T>
  static __device__ __forceinline__ void B(T *out, const T *Q, int d) {
    T a = ncp_a<T>(d);
#pragma unroll
    for (int i = 0; i < 9; i++)
      out[i] = T(0.0);
    out[4] = a * Q[0];
    out[5] = a * T(0.2);
    out[7] = a * T(0.2);
    out[8] = a * Q[0];
  }
  template <class T>
  static __device__ __forceinline__ void S(T *out, const T *Q) {
    out[0] = T(0.0);
    out[1] = T(0.1) * (Q[2] - Q[1]);
    out[2] = T(-0.1) * (Q[1] + Q[2]);
  }
};

struct Burgers2 {
  static constexpr int V = 1, NDIM = 1;
  static constexpr bool HAS_F = true, HAS_B = false, HAS_S = false;
  static constexpr bool SECOND_ORDER = true, HAS_FP32 = true;
  template <class T>
  static __device__ __forceinline__ void F(T *out, const T *Q, const T *dQ, int d) {
    out[0] = ncp_a<T>(d) * (T(0.5) * Q[0] * Q[0]) - T(0.01) * dQ[d];
  }
  template <class T> static __device__ __forceinline__ void B(T *, const T *, int) {}
  template <class T> static __device__ __forceinline__ void S(T *, const T *) {}
};

} // namespace pypde
