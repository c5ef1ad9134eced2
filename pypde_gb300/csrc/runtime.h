// runtime.h -- host runtime of the ADER-WENO library: kernel sets per
// (system, order), the step driver and the stage launchers.
#pragma once

#include "batch.cuh"
#include "mlp.cuh"

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
  // batched launches over many problems of this order (batch.cuh)
  KFunc kb_cfl, kb_predictor, kb_newton, kb_faces[3], kb_centers, kb_gather;
  // learned warm start (k_mlp_guess, batched kb_mlp_guess); guess_k1 == 0:
  // not available
  KFunc guess, kb_guess;
  size_t guess_smem = 0;
  int guess_k1 = 0, guess_no = 0, guess_feat = 0;
  // Rusanov faces in two launches (k_faces_pre, k_faces_eig) through a
  // record buffer of face_rec doubles per face point; face_rec == 0: the
  // one-launch k_faces only
  KFunc faces_pre, faces_eig;
  int face_rec = 0;
  KFunc kb_faces_pre, kb_faces_eig; // their batched forms
};

struct SystemDesc {
  std::string name;
  int ndim = 0, V = 0;
  bool has_F = false, has_B = false, has_S = false, second_order = false;
  KernelSet sets[MAXN + 1];
  bool have[MAXN + 1] = {};
  void *module = nullptr; // CUmodule of a run-time compiled system
};

// Built-in systems, registered by the instantiation units (one order per
// unit, merged by name and dimension).
void register_builtin(const SystemDesc &d);
const SystemDesc *find_builtin(const std::string &name, int ndim);

// Host description of a trained warm-start network (FP32 arrays; weights
// row-major [out][in], W1 [128][k1], W2 [128][128], W3 [no][128]).
struct WarmStartDesc {
  int device = 0;
  int k1 = 0, no = 0, tau_var = -1;
  const float *W1, *b1, *W2, *b2, *W3, *b3;
  const float *x_mean, *x_scale, *y_mean, *y_scale;
};

// A network resident on one device (BF16 weights, FP32 the rest).
struct WarmStart {
  int device = 0;
  void *mem = nullptr;
  MlpModel model;
};

int warm_start_create(const WarmStartDesc &d, WarmStart **out);
void warm_start_free(WarmStart *ws);
int mlp_gemm(const float *A, long long sam, long long sak, const float *B,
             long long sbk, long long sbn, float *C, int M, int N, int K,
             int splits, float *work, const float *bias, float *act,
             cudaStream_t s);
int mlp_silu_grad(const float *dA, const float *Z, float *dZ, long long n,
                  cudaStream_t s);
int mlp_colsum(const float *X, int M, int N, float *out, cudaStream_t s);

// Sampling of (w, converged qh, dt) from the first `steps` steps of a run,
// per_step cells per step, every stride-th reconstruction cell.
struct HarvestArgs {
  int steps = 0;
  long long per_step = 0, stride = 1;
  double *w = nullptr, *qh = nullptr, *dt = nullptr; // host outputs
};

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
  int strips = 0; // predictor strips overlapped with faces; 0 -> automatic
  bool profile = false;
  bool useF = true, useB = true, useS = true;
  const WarmStart *warm = nullptr;    // learned warm start of the Newton predictor
  bool mixed = false;                 // FP32 Newton sweeps before the FP64 ones
  const HarvestArgs *harvest = nullptr;
};

struct Stats {
  long long steps = 0;
  double t_final = 0;
  unsigned long long pred_iters = 0;
  int pred_max_iters = 0, pred_fail = 0, nan_found = 0;
  unsigned long long pred_fallbacks = 0;
  unsigned long long pred_iters32 = 0;
  double device_seconds = 0;
  long long kernel_launches = 0;
  double stage_seconds[8] = {};
};

void set_error(const std::string &msg);
const char *last_error();

int run_solver(const SystemDesc &sys, const RunArgs &a, Stats *st);

// One problem of a batched run.
struct ProblemSpec {
  double *u = nullptr; // host, in/out, prod(nX) x V
  double tf = 0;
  int nX[3] = {1, 1, 1};
  double dX[3] = {1, 1, 1};
  int bt[3] = {0, 0, 0};
  int N = 2;
  double cfl = 0.9;
};

// Stages of a batched step whose tile shape the autotuner picks.
enum BatchStage {
  BS_BOUNDARIES = 0,
  BS_WENO0,
  BS_WENO1,
  BS_WENO2,
  BS_CFL,
  BS_PREDICTOR,
  BS_FACES,
  BS_CENTERS,
  BS_GATHER,
  BS_GUESS, // the learned warm start, before the predictor
  BS_COUNT
};

struct BatchArgs {
  int np = 0;
  ProblemSpec *probs = nullptr;
  bool stiff = false;
  int flux = 0;
  double newton_tol = 1e-12;
  int device = 0;
  int steps_per_graph = 0;
  long long max_steps = -1; // per problem
  bool autotune = true;
  int per_pop = 1; // tiles per queue pop when not autotuning
  bool mixed = false;                     // FP32 Newton sweeps first
  const WarmStart *warm[MAXN + 1] = {};   // learned warm start per order
};

struct BatchStats {
  long long steps = 0, max_problem_steps = 0;
  double device_seconds = 0;
  long long kernel_launches = 0;
  unsigned long long pred_iters = 0;
  int nan_found = 0;
  int per_pop[BS_COUNT] = {};  // chosen tile shape per stage (order group 0)
  double tune_seconds = 0;
  long long *steps_per_problem = nullptr; // optional outputs, np each
  double *t_per_problem = nullptr;
};

int run_batch(const SystemDesc &sys, const BatchArgs &a, BatchStats *st);
int stage_boundaries(const double *u, const int *nX, int ndim, const int *bt,
                     int N, int V, double *ub);
int stage_weno(const double *ub, const int *nXb, int ndim, int N, int V,
               double *w);
int stage_timestep(const SystemDesc &sys, const double *w, long long nrows,
                   const double *dX, int ndim, int N, double cfl, double tf,
                   double t, long long count, double *dt);
int stage_predictor(const SystemDesc &sys, const double *w, long long nrows,
                    const double *dX, int ndim, int N, bool stiff, double dt,
                    double tol, double *qh, Stats *st,
                    const double *guess = nullptr,
                    const WarmStart *warm = nullptr);
int stage_fv(const SystemDesc &sys, double *u, const double *qh,
             const int *nX, const double *dX, int ndim, int N, int flux,
             double dt);

int measure_fp64(int device, double *tflops);
int measure_dmma(int device, double *tflops);

// Instantiation helper used by the per-system units.
template <class Sys, int N> KernelSet make_kernel_set();

} // namespace pypde
