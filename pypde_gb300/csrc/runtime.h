// runtime.h -- host runtime of the ADER-WENO library: kernel sets per
// (system, order), the step driver and the stage launchers.
#pragma once

#include "kernels.cuh"

#include <cuda_runtime.h>
#include <string>

namespace pypde {

int make_tables(int N, Tables *T);
void make_wprod(const Tables &T, int ndim, double *wprod);

// A kernel: ahead-of-time compiled (function symbol) or loaded from a
// module compiled at run time (CUfunction).
struct KFunc {
  const void *aot = nullptr;
  void *jit = nullptr;
  bool valid() const { return aot || jit; }
};

// Kernels of one (system, order).
struct KernelSet {
  KFunc cfl, predictor, newton, faces, centers, gather;
  KFunc faces_flux[3]; // Rusanov, Roe, Osher
  int pred_threads = 0, pred_cpb = 0;
  size_t pred_smem = 0;
  int newton_threads = 0, newton_cpb = 0;
  size_t newton_smem = 0;
};

struct SystemDesc {
  std::string name;
  int ndim = 0, V = 0;
  bool has_F = false, has_B = false, has_S = false, second_order = false;
  KernelSet sets[MAXN + 1];
  bool have[MAXN + 1] = {};
  void *module = nullptr; // CUmodule of a run-time compiled system
};

// Built-in systems, registered by the instantiation units.
void register_builtin(const SystemDesc &d);
const SystemDesc *find_builtin(const std::string &name, int ndim);

struct RunArgs {
  double *u = nullptr; // host, in/out
  double tf = 0;
  int nX[3] = {1, 1, 1};
  int ndim = 1;
  double dX[3] = {1, 1, 1};
  double cfl = 0.9;
  int bt[3] = {0, 0, 0};
  bool stiff = false;
  int flux = 0;
  int N = 2;
  int ndt = 1;
  double *ret = nullptr; // host, ndt x C x V, may be null
  long long max_steps = -1;
  double newton_tol = 1e-12;
  int device = 0;
  int steps_per_graph = 0;
  bool profile = false;
  bool useF = true, useB = true, useS = true;
};

struct Stats {
  long long steps = 0;
  double t_final = 0;
  unsigned long long pred_iters = 0;
  int pred_max_iters = 0, pred_fail = 0, nan_found = 0;
  double device_seconds = 0;
  long long kernel_launches = 0;
  double stage_seconds[8] = {};
};

void set_error(const std::string &msg);
const char *last_error();

int run_solver(const SystemDesc &sys, const RunArgs &a, Stats *st);
int stage_boundaries(const double *u, const int *nX, int ndim, const int *bt,
                     int N, int V, double *ub);
int stage_weno(const double *ub, const int *nXb, int ndim, int N, int V,
               double *w);
int stage_timestep(const SystemDesc &sys, const double *w, long long nrows,
                   const double *dX, int ndim, int N, double cfl, double tf,
                   double t, long long count, double *dt);
int stage_predictor(const SystemDesc &sys, const double *w, long long nrows,
                    const double *dX, int ndim, int N, bool stiff, double dt,
                    double tol, double *qh, Stats *st);
int stage_fv(const SystemDesc &sys, double *u, const double *qh,
             const int *nX, const double *dX, int ndim, int N, int flux,
             double dt);

int measure_fp64(int device, double *tflops);

// Instantiation helper used by the per-system units.
template <class Sys, int N> KernelSet make_kernel_set();

} // namespace pypde
