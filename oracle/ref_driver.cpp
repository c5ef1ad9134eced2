// ref_driver.cpp -- C shim over the reference library (haranjackson/PyPDE
// src/, compiled from its own sources by oracle/Makefile target `ref`).
//
// TEST INFRASTRUCTURE ONLY: it lets tests/golden/make_golden.py call the
// reference's exported stages with the C test callbacks of
// oracle_systems.c and record their outputs as golden vectors.  It runs in
// the development container only (the reference tree is not on the GPU
// machine).
//
// Stages called (paths relative to the reference project):
//   boundaries             src/grid/boundaries.cpp:25
//   WenoSolver             src/solvers/weno/weno.cpp:7,61
//   TimeStepper::step      src/solvers/stepper.cpp:35
//   DGSolver::predictor    src/solvers/dg/dg.cpp:204
//   FVSolver::apply        src/solvers/fv/fv.cpp:200
//   pde_solver             src/api.cpp:5
//   scaled_nodes/weights, basis_polys, derivative_values, end_values
//                          src/poly/basis.cpp
#include "ader_oracle.h"

#include "api.h"
#include "grid/boundaries.h"
#include "poly/basis.h"
#include "eigs/system.h"
#include "solvers/fv/fluxes.h"
#include "solvers/fv/fv.h"
#include "solvers/stepper.h"
#include "solvers/weno/weno.h"
#include "types.h"
#ifdef REF_TIGHT
#include "dg.h" // the tolerance-tightened copy in _ref/patched
#else
#include "solvers/dg/dg.h"
#endif

#include <cstdio>
#include <cstring>
#include <unistd.h>

namespace {
struct Sys {
  ora_flux_fn F;
  ora_ncp_fn B;
  ora_src_fn S;
  int V;
  int so;
};
int lookup(const char *name, int ndim, Sys *s) {
  return ora_system_lookup(name, ndim, &s->V, &s->F, &s->B, &s->S, &s->so);
}
// The reference prints progress to stdout every step; keep it quiet.
struct Quiet {
  int saved;
  Quiet() {
    fflush(stdout);
    saved = dup(1);
    FILE *f = fopen("/dev/null", "w");
    dup2(fileno(f), 1);
    fclose(f);
  }
  ~Quiet() {
    fflush(stdout);
    dup2(saved, 1);
    close(saved);
  }
};
} // namespace

extern "C" {

int ref_tables(int N, double *nodes, double *wghts, double *dervals,
               double *endvals) {
  Vec x = scaled_nodes(N), w = scaled_weights(N);
  std::vector<poly> basis = basis_polys(N);
  Mat D = derivative_values(basis, x);
  Mat E = end_values(basis);
  for (int i = 0; i < N; i++) {
    nodes[i] = x(i);
    wghts[i] = w(i);
    for (int j = 0; j < N; j++)
      dervals[i * N + j] = D(i, j);
    endvals[i] = E(0, i);
    endvals[N + i] = E(1, i);
  }
  return 0;
}

int ref_boundaries(const double *u, const int *nX, int ndim, const int *bt,
                   int N, int V, double *ub) {
  iVec nx(ndim), b(ndim);
  long nc = 1;
  for (int d = 0; d < ndim; d++) {
    nx(d) = nX[d];
    b(d) = bt[d];
    nc *= nX[d];
  }
  Mat um = Eigen::Map<const Mat>(u, nc, V);
  Mat r = boundaries(um, nx, b, N);
  memcpy(ub, r.data(), sizeof(double) * r.size());
  return 0;
}

// Same contract as the reference's weno_solver (src/api.cpp:32-48).
int ref_weno(const double *ub, const int *nXb, int ndim, int N, int V,
             double *w) {
  iVec nx(ndim);
  long nc = 1;
  for (int d = 0; d < ndim; d++) {
    nx(d) = nXb[d];
    nc *= nXb[d];
  }
  WenoSolver ws(nx, N, V);
  Mat um = Eigen::Map<const Mat>(ub, nc, V);
  Mat r = ws.reconstruction(um);
  memcpy(w, r.data(), sizeof(double) * r.size());
  return 0;
}

double ref_timestep(const char *sys, const double *w, long nrows,
                    const double *dX, int ndim, int N, double CFL, double tf,
                    double t, int count) {
  Sys s;
  if (lookup(sys, ndim, &s))
    return -1;
  Vec dx(ndim);
  for (int d = 0; d < ndim; d++)
    dx(d) = dX[d];
  TimeStepper ts(s.F, s.B, dx, N, s.V, CFL, tf, s.so);
  Mat wm = Eigen::Map<const Mat>(w, nrows, s.V);
  return ts.step(wm, t, count);
}

int ref_predictor(const char *sys, const double *w, long nrows,
                  const double *dX, int ndim, int N, int stiff, double dt,
                  double *qh) {
  Sys s;
  if (lookup(sys, ndim, &s))
    return -1;
  Vec dx(ndim);
  for (int d = 0; d < ndim; d++)
    dx(d) = dX[d];
  DGSolver dg(s.F, s.B, s.S, dx, stiff, N, s.V);
  Mat wm = Eigen::Map<const Mat>(w, nrows, s.V);
  Mat r = dg.predictor(wm, dt);
  memcpy(qh, r.data(), sizeof(double) * r.size());
  return 0;
}

int ref_fv(const char *sys, double *u, const double *qh, const int *nX,
           const double *dX, int ndim, int N, int flux, double dt) {
  Sys s;
  if (lookup(sys, ndim, &s))
    return -1;
  iVec nx(ndim);
  Vec dx(ndim);
  long nc = 1, nw = 1;
  for (int d = 0; d < ndim; d++) {
    nx(d) = nX[d];
    dx(d) = dX[d];
    nc *= nX[d];
    nw *= nX[d] + 2;
  }
  int Nd = 1;
  for (int d = 0; d < ndim; d++)
    Nd *= N;
  FVSolver fv(s.F, s.B, s.S, nx, dx, flux, N, s.V, s.so);
  Mat um = Eigen::Map<Mat>(u, nc, s.V);
  Mat qm = Eigen::Map<const Mat>(qh, nw * N * Nd, s.V);
  fv.apply(um, qm, dt);
  memcpy(u, um.data(), sizeof(double) * um.size());
  return 0;
}

// pde_solver through the reference's own C ABI (src/api.cpp:5-30).
int ref_pde_solver(const char *sys, double *u, double tf, int *nX, int ndim,
                   double *dX, double CFL, int *bt, int stiff, int flux, int N,
                   int ndt, double *ret, int nThreads) {
  Sys s;
  if (lookup(sys, ndim, &s))
    return -1;
  Quiet q;
  pde_solver(s.F, s.B, s.S, s.F != nullptr, s.B != nullptr, s.S != nullptr, u,
             tf, nX, ndim, dX, CFL, bt, stiff, flux, N, s.V, ndt, s.so, ret,
             nThreads);
  return 0;
}

// Time of each of the first K steps as the reference's loop computes it
// (iterator.cpp:99-132 with one slab, which is bit-identical to any slab
// count): lets a caller set tf to t_K so pde_solver runs exactly K steps.
int ref_step_times(const char *sys, const double *u0, int *nX, int ndim,
                   double *dX, double CFL, int *bt, int stiff, int flux, int N,
                   double tf, int K, double *times) {
  Sys s;
  if (lookup(sys, ndim, &s))
    return -1;
  iVec nx(ndim), b(ndim), nxb(ndim);
  Vec dx(ndim);
  long nc = 1;
  for (int d = 0; d < ndim; d++) {
    nx(d) = nX[d];
    b(d) = bt[d];
    nxb(d) = nX[d] + 2 * N;
    dx(d) = dX[d];
    nc *= nX[d];
  }
  Mat u = Eigen::Map<const Mat>(u0, nc, s.V);
  WenoSolver ws(nxb, N, s.V);
  TimeStepper ts(s.F, s.B, dx, N, s.V, CFL, tf, s.so);
  DGSolver dg(s.F, s.B, s.S, dx, stiff, N, s.V);
  FVSolver fv(s.F, s.B, s.S, nx, dx, flux, N, s.V, s.so);
  double t = 0;
  for (int k = 0; k < K && t < tf; k++) {
    Mat ub = boundaries(u, nx, b, N);
    Mat w = ws.reconstruction(ub);
    double dt = ts.step(w, t, k);
    Mat qh = dg.predictor(w, dt);
    fv.apply(u, qh, dt);
    t += dt;
    times[k] = t;
  }
  return 0;
}
}

extern "C" {
// max |eig| of the FD Jacobian + B at one state (src/eigs/system.cpp:45-51)
double ref_max_abs_eigs(const char *sys, int ndim, double *q, double *dq,
                        int d) {
  Sys s;
  if (lookup(sys, ndim, &s))
    return -1;
  Eigen::Map<Vec> qv(q, s.V);
  Eigen::Map<Mat> dqm(dq, ndim, s.V);
  return max_abs_eigs(s.F, s.B, qv, dqm, d);
}
// the FD Jacobian + B itself (src/eigs/system.cpp:6-26)
int ref_system_matrix(const char *sys, int ndim, double *q, double *dq, int d,
                      double *M) {
  Sys s;
  if (lookup(sys, ndim, &s))
    return -1;
  Eigen::Map<Vec> qv(q, s.V);
  Eigen::Map<Mat> dqm(dq, ndim, s.V);
  Mat m = system_matrix(s.F, s.B, qv, dqm, d);
  memcpy(M, m.data(), sizeof(double) * m.size());
  return 0;
}
}

extern "C" {
// Numerical flux D(qL,qR)+F(qL)+F(qR) of src/solvers/fv/fluxes.cpp:80-101
// (flux 0 Rusanov, 1 Roe, 2 Osher) and the B path integral of :103-117, at
// one face point, through the reference's FluxGenerator.
int ref_flux(const char *sys, int ndim, int N, double *qL, double *qR,
             double *dqL, double *dqR, int d, int flux, double *f, double *b) {
  Sys s;
  if (lookup(sys, ndim, &s))
    return -1;
  Vec nodes = scaled_nodes(N), wghts = scaled_weights(N);
  Vec dx = Vec::Ones(ndim);
  FluxGenerator fg(s.F, s.B, nodes, wghts, dx, s.V, flux, ndim);
  Eigen::Map<Vec> ql(qL, s.V), qr(qR, s.V);
  Eigen::Map<Mat> dql(dqL, ndim, s.V), dqr(dqR, ndim, s.V);
  Vec fv = Vec::Zero(s.V), bv = Vec::Zero(s.V);
  if (s.F)
    fg.flux(fv, ql, qr, dql, dqr, d, s.so);
  if (s.B)
    fg.Bint(bv, ql, qr, d);
  for (int i = 0; i < s.V; i++) {
    f[i] = fv(i);
    b[i] = bv(i);
  }
  return 0;
}
}
