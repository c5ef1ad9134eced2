// The device face-flux functions of pypde_gb300/csrc/kernels.cuh (Rusanov,
// Roe, Osher, the B path integral, with the FD Jacobians and eigensolvers
// they call) compiled as host C++, for a CPU test that compares them bit
// for bit with the C restatement.  The shims stand in for the CUDA
// qualifiers, built-in variables, barriers and atomics: the kernel bodies
// that use those are templates that this unit never instantiates, and the
// flux functions it does instantiate use only IEEE arithmetic and fma.
#include <cmath>
#include <cstring>

#define __device__
#define __host__
#define __global__
#define __shared__
#define __grid_constant__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __launch_bounds__(...)

struct HostDim3 {
  unsigned x, y, z;
};
static HostDim3 threadIdx, blockIdx, blockDim, gridDim;
static inline void __syncthreads() {}
static inline int __syncthreads_and(int p) { return p; }
static inline int __syncthreads_or(int p) { return p; }
static inline void __syncwarp(unsigned = 0xffffffffu) {}
static inline unsigned __float_as_uint(float x) {
  unsigned r;
  std::memcpy(&r, &x, sizeof r);
  return r;
}
template <class T> static inline T max(T a, T b) { return a > b ? a : b; }
template <class T> static inline T __shfl_down_sync(unsigned, T v, int) {
  return v;
}
template <class T> static inline T atomicAdd(T *a, T v) {
  const T o = *a;
  *a = o + v;
  return o;
}
template <class T> static inline T atomicMax(T *a, T v) {
  const T o = *a;
  if (v > o)
    *a = v;
  return o;
}
template <class T> static inline T atomicOr(T *a, T v) {
  const T o = *a;
  *a = o | v;
  return o;
}
static inline long long __double_as_longlong(double x) {
  long long r;
  std::memcpy(&r, &x, sizeof r);
  return r;
}
static inline double __longlong_as_double(long long x) {
  double r;
  std::memcpy(&r, &x, sizeof r);
  return r;
}

using std::fabs;
using std::fma;
using std::fmax;
using std::sqrt;

#include "../pypde_gb300/csrc/kernels.cuh"
#include "../pypde_gb300/csrc/systems.cuh"

namespace {
using namespace pypde;

template <class Sys, int N>
void flux_at(int flux, double *qL, double *qR, double *dqL, double *dqR, int d,
             const Tables &T, double *f, double *b) {
  constexpr int V = Sys::V;
  for (int v = 0; v < V; v++)
    f[v] = b[v] = 0.0;
  const double dXd = 1.0; // unit cells, as in the restatement's test hook
  if (Sys::HAS_F) {
    if (flux == 0)
      rusanov_flux<Sys, N>(f, qL, qR, dqL, dqR, d, dXd);
    else if (flux == 1)
      eig_flux<Sys, N, 1>(f, qL, qR, dqL, dqR, d, dXd, T);
    else
      eig_flux<Sys, N, 2>(f, qL, qR, dqL, dqR, d, dXd, T);
  }
  if (Sys::HAS_B)
    bint<Sys, N>(b, qL, qR, d, T);
}

template <class Sys>
int flux_n(int N, int flux, double *qL, double *qR, double *dqL, double *dqR,
           int d, const Tables &T, double *f, double *b) {
  if (N == 1)
    flux_at<Sys, 1>(flux, qL, qR, dqL, dqR, d, T, f, b);
  else if (N == 2)
    flux_at<Sys, 2>(flux, qL, qR, dqL, dqR, d, T, f, b);
  else if (N == 3)
    flux_at<Sys, 3>(flux, qL, qR, dqL, dqR, d, T, f, b);
  else
    return -1;
  return 0;
}
} // namespace

// The numerical flux f = D(qL, qR) + F(qL) + F(qR) and the B path integral
// b at one face point of a built-in system, through the device code, with
// the order-N Gauss-Legendre nodes and weights given; -1 for an unknown
// system or order.
extern "C" int host_face_flux(const char *name, int ndim, int N, double *qL,
                              double *qR, double *dqL, double *dqR, int d,
                              int flux, const double *nodes,
                              const double *wghts, double *f, double *b) {
  Tables T;
  std::memset(&T, 0, sizeof T);
  if (N < 1 || N > MAXN)
    return -1;
  T.N = N;
  for (int i = 0; i < N; i++) {
    T.nodes[i] = nodes[i];
    T.wghts[i] = wghts[i];
  }
  if (!std::strcmp(name, "euler")) {
    if (ndim == 1)
      return flux_n<Euler<1>>(N, flux, qL, qR, dqL, dqR, d, T, f, b);
    if (ndim == 2)
      return flux_n<Euler<2>>(N, flux, qL, qR, dqL, dqR, d, T, f, b);
    if (ndim == 3)
      return flux_n<Euler<3>>(N, flux, qL, qR, dqL, dqR, d, T, f, b);
  } else if (!std::strcmp(name, "cattaneo")) {
    if (ndim == 2)
      return flux_n<Cattaneo<2>>(N, flux, qL, qR, dqL, dqR, d, T, f, b);
    if (ndim == 3)
      return flux_n<Cattaneo<3>>(N, flux, qL, qR, dqL, dqR, d, T, f, b);
  } else if (!std::strcmp(name, "ncp")) {
    if (ndim == 1)
      return flux_n<Ncp<1>>(N, flux, qL, qR, dqL, dqR, d, T, f, b);
    if (ndim == 2)
      return flux_n<Ncp<2>>(N, flux, qL, qR, dqL, dqR, d, T, f, b);
  } else if (!std::strcmp(name, "burgers2")) {
    if (ndim == 1)
      return flux_n<Burgers2>(N, flux, qL, qR, dqL, dqR, d, T, f, b);
  }
  return -1;
}
