// api.cpp -- the extern "C" entry points of include/pypde_gb300.h.
#include "../../include/pypde_gb300.h"
#include "runtime.h"

#include <cstring>
#include <new>
#include <vector>

struct pypde_system {
  const pypde::SystemDesc *desc;
  pypde::SystemDesc *owned; // run-time compiled systems
};

struct pypde_warm_start {
  pypde::WarmStart *ws;
  int N, V, ndim;
};

namespace pypde {
int compile_system(const char *src, const char *name, int ndim, int V,
                   int has_F, int has_B, int has_S, int second_order,
                   SystemDesc **out);
void release_system(SystemDesc *d);
} // namespace pypde

using namespace pypde;

static int resolve(const pypde_system *F, const pypde_system *B,
                   const pypde_system *S, const SystemDesc **out) {
  const pypde_system *h = F ? F : (B ? B : S);
  if (!h) {
    set_error("no callback system given");
    return PYPDE_ERR_ARG;
  }
  if ((F && F->desc != h->desc) || (B && B->desc != h->desc) ||
      (S && S->desc != h->desc)) {
    set_error("F, B and S must come from one callback system");
    return PYPDE_ERR_ARG;
  }
  *out = h->desc;
  return PYPDE_OK;
}

extern "C" {

int pypde_system_builtin(const char *name, int ndim, pypde_system **out) {
  if (!name || !out) {
    set_error("null argument");
    return PYPDE_ERR_ARG;
  }
  const SystemDesc *d = find_builtin(name, ndim);
  if (!d) {
    set_error(std::string("no built-in system '") + name + "' for ndim " +
              std::to_string(ndim));
    return PYPDE_ERR_ARG;
  }
  *out = new (std::nothrow) pypde_system{d, nullptr};
  return *out ? PYPDE_OK : PYPDE_ERR_ARG;
}

int pypde_system_compile(const char *src, const char *name, int ndim, int V,
                         int has_F, int has_B, int has_S, int second_order,
                         pypde_system **out) {
  if (!src || !out) {
    set_error("null argument");
    return PYPDE_ERR_ARG;
  }
  SystemDesc *d = nullptr;
  int rc = compile_system(src, name ? name : "user", ndim, V, has_F, has_B,
                          has_S, second_order, &d);
  if (rc)
    return rc;
  *out = new (std::nothrow) pypde_system{d, d};
  if (!*out) {
    release_system(d);
    set_error("out of host memory");
    return PYPDE_ERR_ARG;
  }
  return PYPDE_OK;
}

int pypde_system_info(const pypde_system *s, int *V, int *ndim, int *has_F,
                      int *has_B, int *has_S, int *second_order) {
  if (!s) {
    set_error("null system");
    return PYPDE_ERR_ARG;
  }
  if (V)
    *V = s->desc->V;
  if (ndim)
    *ndim = s->desc->ndim;
  if (has_F)
    *has_F = s->desc->has_F;
  if (has_B)
    *has_B = s->desc->has_B;
  if (has_S)
    *has_S = s->desc->has_S;
  if (second_order)
    *second_order = s->desc->second_order;
  return PYPDE_OK;
}

void pypde_system_free(pypde_system *s) {
  if (!s)
    return;
  if (s->owned)
    release_system(s->owned);
  delete s;
}

static int run_ex(const pypde_system *sys, const RunArgs &a,
                  pypde_stats *stats);

int pde_solver_ex(const pypde_system *sys, bool useF, bool useB, bool useS,
                  double *u, double tf, const int *nX, int ndim,
                  const double *dX, double CFL, const int *boundaryTypes,
                  bool STIFF, int FLUX, int N, int ndt, double *ret,
                  const pypde_options *opt, pypde_stats *stats) {
  if (!sys || !u || !nX || !dX || !boundaryTypes || ndim < 1 || ndim > 3) {
    set_error("invalid arguments");
    return PYPDE_ERR_ARG;
  }
  RunArgs a;
  a.u = u;
  a.tf = tf;
  a.ndim = ndim;
  for (int d = 0; d < ndim; d++) {
    a.nX[d] = nX[d];
    a.dX[d] = dX[d];
    a.bt[d] = boundaryTypes[d];
    if (a.bt[d] != 0 && a.bt[d] != 1) {
      set_error("boundaryTypes must be 0 (transmissive) or 1 (periodic)");
      return PYPDE_ERR_ARG;
    }
  }
  a.cfl = CFL;
  a.stiff = STIFF;
  a.flux = FLUX;
  a.N = N;
  a.ndt = ndt;
  a.ret = ret;
  a.useF = useF;
  a.useB = useB;
  a.useS = useS;
  if (opt) {
    a.max_steps = opt->max_steps > 0 ? opt->max_steps : -1;
    if (opt->newton_tol > 0)
      a.newton_tol = opt->newton_tol;
    a.device = opt->device;
    a.steps_per_graph = opt->steps_per_graph;
    a.profile = opt->profile_stages != 0;
    if (opt->strips < 0 || opt->strips > 32) {
      set_error("strips must be 0 (automatic) to 32");
      return PYPDE_ERR_ARG;
    }
    a.strips = opt->strips;
    if (opt->warm_start) {
      const pypde_warm_start *w = opt->warm_start;
      if (w->N != N || w->V != sys->desc->V || w->ndim != ndim) {
        set_error("warm start was built for another system, order or ndim");
        return PYPDE_ERR_ARG;
      }
      a.warm = w->ws;
    }
    a.mixed = opt->mixed_precision != 0;
  }
  if (a.mixed) {
    if (!STIFF) {
      set_error("mixed_precision applies to the stiff (Newton) predictor");
      return PYPDE_ERR_ARG;
    }
    if (sys->desc->module) {
      set_error("mixed_precision needs FP32 callbacks: built-in systems only");
      return PYPDE_ERR_UNSUPPORTED;
    }
  }
  return run_ex(sys, a, stats);
}

static int run_ex(const pypde_system *sys, const RunArgs &a,
                  pypde_stats *stats) {
  Stats st;
  int rc = run_solver(*sys->desc, a, &st);
  if (stats) {
    stats->steps = st.steps;
    stats->t_final = st.t_final;
    stats->pred_iters = st.pred_iters;
    stats->pred_max_iters = st.pred_max_iters;
    stats->pred_fail = st.pred_fail;
    stats->nan_found = st.nan_found;
    stats->device_seconds = st.device_seconds;
    stats->kernel_launches = st.kernel_launches;
    for (int i = 0; i < 8; i++)
      stats->stage_seconds[i] = st.stage_seconds[i];
    stats->pred_fallbacks = st.pred_fallbacks;
    stats->pred_iters32 = st.pred_iters32;
  }
  return rc;
}

int pde_solver(const pypde_system *F, const pypde_system *B,
               const pypde_system *S, bool useF, bool useB, bool useS,
               double *u, double tf, int *nX, int ndim, double *dX, double CFL,
               int *boundaryTypes, bool STIFF, int FLUX, int N, int V, int ndt,
               bool secondOrder, double *ret, int nThreads) {
  (void)nThreads;
  const SystemDesc *d;
  int rc = resolve(useF ? F : nullptr, useB ? B : nullptr, useS ? S : nullptr,
                   &d);
  if (rc)
    return rc;
  if (V != d->V || secondOrder != d->second_order) {
    set_error("V or secondOrder does not match the callback system");
    return PYPDE_ERR_ARG;
  }
  pypde_system h{d, nullptr};
  return pde_solver_ex(&h, useF, useB, useS, u, tf, nX, ndim, dX, CFL,
                       boundaryTypes, STIFF, FLUX, N, ndt, ret, nullptr,
                       nullptr);
}

int weno_solver(double *ret, double *u, int *nX, int ndim, int N, int V) {
  if (!ret || !u || !nX) {
    set_error("null argument");
    return PYPDE_ERR_ARG;
  }
  return stage_weno(u, nX, ndim, N, V, ret);
}

int pypde_boundaries(const double *u, const int *nX, int ndim,
                     const int *boundaryTypes, int N, int V, double *ub) {
  if (!u || !nX || !boundaryTypes || !ub) {
    set_error("null argument");
    return PYPDE_ERR_ARG;
  }
  return stage_boundaries(u, nX, ndim, boundaryTypes, N, V, ub);
}

int pypde_timestep(const pypde_system *sys, const double *w, long long nrows,
                   const double *dX, int ndim, int N, double CFL, double tf,
                   double t, long long count, double *dt_out) {
  if (!sys || !w || !dX || !dt_out) {
    set_error("null argument");
    return PYPDE_ERR_ARG;
  }
  return stage_timestep(*sys->desc, w, nrows, dX, ndim, N, CFL, tf, t, count,
                        dt_out);
}

int pypde_predictor(const pypde_system *sys, const double *w, long long nrows,
                    const double *dX, int ndim, int N, bool STIFF, double dt,
                    double newton_tol, double *qh, pypde_stats *stats) {
  if (!sys || !w || !dX || !qh) {
    set_error("null argument");
    return PYPDE_ERR_ARG;
  }
  Stats st;
  int rc = stage_predictor(*sys->desc, w, nrows, dX, ndim, N, STIFF, dt,
                           newton_tol > 0 ? newton_tol : 1e-12, qh, &st);
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->pred_iters = st.pred_iters;
    stats->pred_max_iters = st.pred_max_iters;
    stats->pred_fail = st.pred_fail;
  }
  return rc;
}

// ---------------------------------------------------------------- batch

int pde_solver_batch(const pypde_system *sys, bool STIFF, int FLUX, int nprob,
                     pypde_problem *problems, const pypde_batch_options *opt,
                     pypde_batch_stats *stats, long long *steps_out,
                     double *t_out) {
  if (!sys || nprob < 1 || !problems || FLUX < 0 || FLUX > 2) {
    set_error("invalid arguments");
    return PYPDE_ERR_ARG;
  }
  std::vector<ProblemSpec> ps(nprob);
  for (int p = 0; p < nprob; p++) {
    ps[p].u = problems[p].u;
    ps[p].tf = problems[p].tf;
    ps[p].N = problems[p].N;
    ps[p].cfl = problems[p].cfl;
    for (int d = 0; d < 3; d++) {
      ps[p].nX[d] = d < sys->desc->ndim ? problems[p].nX[d] : 1;
      ps[p].dX[d] = d < sys->desc->ndim ? problems[p].dX[d] : 1.0;
      ps[p].bt[d] = d < sys->desc->ndim ? problems[p].boundaryTypes[d] : 0;
    }
  }
  BatchArgs a;
  a.np = nprob;
  a.probs = ps.data();
  a.stiff = STIFF;
  a.flux = FLUX;
  if (opt) {
    a.max_steps = opt->max_steps > 0 ? opt->max_steps : -1;
    if (opt->newton_tol > 0)
      a.newton_tol = opt->newton_tol;
    a.device = opt->device;
    a.steps_per_graph = opt->steps_per_graph;
    a.autotune = opt->autotune != 0;
    a.per_pop = opt->per_pop >= 0 ? opt->per_pop : 1;
    a.mixed = opt->mixed_precision != 0;
    for (int n = 1; n <= 3 && n <= MAXN; n++) {
      const pypde_warm_start *w = opt->warm_start[n];
      if (!w)
        continue;
      if (w->N != n || w->V != sys->desc->V || w->ndim != sys->desc->ndim) {
        set_error("batch warm_start[" + std::to_string(n) +
                  "] was built for another system, order or ndim");
        return PYPDE_ERR_ARG;
      }
      a.warm[n] = w->ws;
    }
    if (opt->warm_start[0]) {
      set_error("batch warm_start is indexed by order: entry 0 must be NULL");
      return PYPDE_ERR_ARG;
    }
  }
  if (a.mixed) {
    if (!STIFF) {
      set_error("mixed_precision applies to the stiff (Newton) predictor");
      return PYPDE_ERR_ARG;
    }
    if (sys->desc->module) {
      set_error("mixed_precision needs FP32 callbacks: built-in systems only");
      return PYPDE_ERR_UNSUPPORTED;
    }
  }
  BatchStats st;
  st.steps_per_problem = steps_out;
  st.t_per_problem = t_out;
  int rc = run_batch(*sys->desc, a, &st);
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->steps = st.steps;
    stats->max_problem_steps = st.max_problem_steps;
    stats->device_seconds = st.device_seconds;
    stats->kernel_launches = st.kernel_launches;
    stats->pred_iters = st.pred_iters;
    stats->nan_found = st.nan_found;
    for (int i = 0; i < PYPDE_BATCH_STAGES && i < BS_COUNT; i++)
      stats->per_pop[i] = st.per_pop[i];
    stats->tune_seconds = st.tune_seconds;
  }
  return rc;
}

// ---------------------------------------------------------------- warm start

static int warm_shape(const pypde_system *sys, int N, int *feat, int *k1,
                      int *no) {
  if (!sys || N < 1 || N > MAXN) {
    set_error("invalid arguments");
    return PYPDE_ERR_ARG;
  }
  const SystemDesc &d = *sys->desc;
  int Nd = 1;
  for (int i = 0; i < d.ndim; i++)
    Nd *= N;
  int f = d.V + Nd * d.V + 2, k = (f + 15) / 16 * 16,
      o = (N * Nd * d.V + 7) / 8 * 8;
  if (feat)
    *feat = f;
  if (k1)
    *k1 = k;
  if (no)
    *no = o;
  if (!d.has_S || k > 128 || o > 256) {
    set_error("no warm-start network for system " + d.name +
              " at this order (needs a source term, <= 128 features and "
              "<= 256 outputs)");
    return PYPDE_ERR_UNSUPPORTED;
  }
  return PYPDE_OK;
}

int pypde_warm_start_shape(const pypde_system *sys, int N, int *feat, int *k1,
                           int *no) {
  return warm_shape(sys, N, feat, k1, no);
}

int pypde_warm_start_create(const pypde_system *sys, int N, int device,
                            const float *W1, const float *b1, const float *W2,
                            const float *b2, const float *W3, const float *b3,
                            const float *x_mean, const float *x_scale,
                            const float *y_mean, const float *y_scale,
                            int tau_var, pypde_warm_start **out) {
  int k1 = 0, no = 0;
  int rc = warm_shape(sys, N, nullptr, &k1, &no);
  if (rc)
    return rc;
  if (!W1 || !b1 || !W2 || !b2 || !W3 || !b3 || !x_mean || !x_scale ||
      !y_mean || !y_scale || !out || tau_var >= sys->desc->V) {
    set_error("invalid arguments");
    return PYPDE_ERR_ARG;
  }
  WarmStartDesc d;
  d.device = device;
  d.k1 = k1;
  d.no = no;
  d.tau_var = tau_var < 0 ? -1 : tau_var;
  d.W1 = W1;
  d.b1 = b1;
  d.W2 = W2;
  d.b2 = b2;
  d.W3 = W3;
  d.b3 = b3;
  d.x_mean = x_mean;
  d.x_scale = x_scale;
  d.y_mean = y_mean;
  d.y_scale = y_scale;
  WarmStart *ws = nullptr;
  rc = warm_start_create(d, &ws);
  if (rc)
    return rc == -1 ? PYPDE_ERR_ARG : PYPDE_ERR_CUDA;
  pypde_warm_start *h = new (std::nothrow) pypde_warm_start;
  if (!h) {
    warm_start_free(ws);
    set_error("out of host memory");
    return PYPDE_ERR_ARG;
  }
  h->ws = ws;
  h->N = N;
  h->V = sys->desc->V;
  h->ndim = sys->desc->ndim;
  *out = h;
  return PYPDE_OK;
}

int pypde_warm_start_free(pypde_warm_start *ws) {
  if (ws) {
    warm_start_free(ws->ws);
    delete ws;
  }
  return PYPDE_OK;
}

int pypde_predictor_guess(const pypde_system *sys, const double *w,
                          long long nrows, const double *dX, int ndim, int N,
                          double dt, double newton_tol, const double *guess,
                          const pypde_warm_start *warm, double *qh,
                          pypde_stats *stats) {
  if (!sys || !w || !dX || !qh || (!guess && !warm) || (guess && warm)) {
    set_error("invalid arguments (give exactly one of guess and warm)");
    return PYPDE_ERR_ARG;
  }
  if (warm && (warm->N != N || warm->V != sys->desc->V || warm->ndim != ndim)) {
    set_error("warm start was built for another system, order or ndim");
    return PYPDE_ERR_ARG;
  }
  Stats st;
  int rc = stage_predictor(*sys->desc, w, nrows, dX, ndim, N, true, dt,
                           newton_tol > 0 ? newton_tol : 1e-12, qh, &st, guess,
                           warm ? warm->ws : nullptr);
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->pred_iters = st.pred_iters;
    stats->pred_max_iters = st.pred_max_iters;
    stats->pred_fail = st.pred_fail;
    stats->pred_fallbacks = st.pred_fallbacks;
  }
  return rc;
}

int pypde_harvest(const pypde_system *sys, double *u, double tf,
                  const int *nX, int ndim, const double *dX, double CFL,
                  const int *boundaryTypes, bool STIFF, int N, int steps,
                  long long per_step, long long stride, double *w_out,
                  double *qh_out, double *dt_out, const pypde_options *opt,
                  pypde_stats *stats) {
  if (!sys || !u || !nX || !dX || !boundaryTypes || ndim < 1 || ndim > 3 ||
      steps < 1 || per_step < 1 || stride < 1 || !w_out || !qh_out ||
      !dt_out) {
    set_error("invalid arguments");
    return PYPDE_ERR_ARG;
  }
  RunArgs a;
  a.u = u;
  a.tf = tf;
  a.ndim = ndim;
  for (int d = 0; d < ndim; d++) {
    a.nX[d] = nX[d];
    a.dX[d] = dX[d];
    a.bt[d] = boundaryTypes[d];
  }
  a.cfl = CFL;
  a.stiff = STIFF;
  a.N = N;
  a.useF = sys->desc->has_F;
  a.useB = sys->desc->has_B;
  a.useS = sys->desc->has_S;
  a.max_steps = steps;
  if (opt) {
    if (opt->newton_tol > 0)
      a.newton_tol = opt->newton_tol;
    a.device = opt->device;
  }
  HarvestArgs h;
  h.steps = steps;
  h.per_step = per_step;
  h.stride = stride;
  h.w = w_out;
  h.qh = qh_out;
  h.dt = dt_out;
  a.harvest = &h;
  return run_ex(sys, a, stats);
}

// ------------------------------------------------------- training kernels

int pypde_mlp_gemm(const float *A, long long sam, long long sak,
                   const float *B, long long sbk, long long sbn, float *C,
                   int M, int N, int K, int splits, float *work,
                   const float *bias, float *act, void *stream) {
  if (!A || !B) {
    set_error("null operand");
    return PYPDE_ERR_ARG;
  }
  int rc = mlp_gemm(A, sam, sak, B, sbk, sbn, C, M, N, K, splits, work, bias,
                    act, (cudaStream_t)stream);
  return rc == 0 ? PYPDE_OK : (rc == -1 ? PYPDE_ERR_ARG : PYPDE_ERR_CUDA);
}

int pypde_mlp_silu_grad(const float *dA, const float *Z, float *dZ,
                        long long n, void *stream) {
  if (!dA || !Z || !dZ) {
    set_error("null operand");
    return PYPDE_ERR_ARG;
  }
  int rc = mlp_silu_grad(dA, Z, dZ, n, (cudaStream_t)stream);
  return rc == 0 ? PYPDE_OK : PYPDE_ERR_CUDA;
}

int pypde_mlp_colsum(const float *X, int M, int N, float *out, void *stream) {
  if (!X || !out) {
    set_error("null operand");
    return PYPDE_ERR_ARG;
  }
  int rc = mlp_colsum(X, M, N, out, (cudaStream_t)stream);
  return rc == 0 ? PYPDE_OK : (rc == -1 ? PYPDE_ERR_ARG : PYPDE_ERR_CUDA);
}

int pypde_fv(const pypde_system *sys, double *u, const double *qh,
             const int *nX, const double *dX, int ndim, int N, int FLUX,
             double dt) {
  if (!sys || !u || !qh || !nX || !dX) {
    set_error("null argument");
    return PYPDE_ERR_ARG;
  }
  return stage_fv(*sys->desc, u, qh, nX, dX, ndim, N, FLUX, dt);
}

int pypde_tables(int N, double *out) {
  Tables T;
  if (!out || make_tables(N, &T)) {
    set_error("invalid order");
    return PYPDE_ERR_ARG;
  }
  double *o = out;
  auto put = [&](const double *p, int n) {
    std::memcpy(o, p, sizeof(double) * n);
    o += n;
  };
  put(T.nodes, N);
  put(T.wghts, N);
  put(T.dervals, N * N);
  put(T.endvals, 2 * N);
  put(T.dgmat, N * N);
  put(T.dgmat_inv, N * N);
  for (int k = 0; k < 4; k++)
    put(T.weno_inv[k], N * N);
  put(T.sig, N * N);
  return PYPDE_OK;
}

int pypde_measure_fp64_peak(int device, double *tflops) {
  if (!tflops) {
    set_error("null argument");
    return PYPDE_ERR_ARG;
  }
  return measure_fp64(device, tflops);
}

int pypde_measure_dmma_peak(int device, double *tflops) {
  if (!tflops) {
    set_error("null argument");
    return PYPDE_ERR_ARG;
  }
  return measure_dmma(device, tflops);
}

const char *pypde_last_error(void) { return last_error(); }

} // extern "C"
