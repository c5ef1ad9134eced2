// The device eigenvalue path (pypde_gb300/csrc/ader_common.cuh with the
// built-in systems of systems.cuh) compiled as host C++, for a CPU test
// that compares it bit for bit with the C restatement.  The shims below
// stand in for the CUDA qualifiers and intrinsics the two headers use; the
// arithmetic is IEEE +, -, *, /, sqrt and fused fma on both targets, so a
// host build gives the device's bits as long as the operation order is the
// same (host -ffp-contract=off, device --fmad=false).
#include <cmath>
#include <cstring>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))

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
static inline unsigned long long atomicMax(unsigned long long *a,
                                           unsigned long long v) {
  const unsigned long long o = *a;
  if (v > o)
    *a = v;
  return o;
}

using std::fabs;
using std::fma;
using std::fmax;
using std::sqrt;

#include "../pypde_gb300/csrc/ader_common.cuh"
#include "../pypde_gb300/csrc/systems.cuh"

namespace {
template <class Sys> double eigs(double *q, double *dq, int d) {
  return pypde::max_abs_eigs<Sys>(q, dq, d);
}
} // namespace

// max|eig| of the system matrix of a built-in system at (q, dq) in
// direction d, through the device code path; NaN for an unknown system.
extern "C" double host_max_abs_eigs(const char *name, int ndim, double *q,
                                    double *dq, int d) {
  using namespace pypde;
  if (!std::strcmp(name, "euler")) {
    if (ndim == 1)
      return eigs<Euler<1>>(q, dq, d);
    if (ndim == 2)
      return eigs<Euler<2>>(q, dq, d);
    if (ndim == 3)
      return eigs<Euler<3>>(q, dq, d);
  } else if (!std::strcmp(name, "cattaneo")) {
    if (ndim == 2)
      return eigs<Cattaneo<2>>(q, dq, d);
    if (ndim == 3)
      return eigs<Cattaneo<3>>(q, dq, d);
  } else if (!std::strcmp(name, "ncp")) {
    if (ndim == 1)
      return eigs<Ncp<1>>(q, dq, d);
    if (ndim == 2)
      return eigs<Ncp<2>>(q, dq, d);
  }
  return std::nan("");
}

// The device FD quotient (fd_step + fd_div) over n pairs: out[i] = x[i] /
// h[i] as the kernels form it.
extern "C" void host_fd_div(const double *x, const double *h, double *out,
                            long n) {
  for (long i = 0; i < n; i++)
    out[i] = pypde::fd_div(x[i], pypde::fd_step(h[i]));
}
