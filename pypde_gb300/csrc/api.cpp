// api.cpp -- the extern "C" entry points of include/pypde_gb300.h.
#include "../../include/pypde_gb300.h"
#include "runtime.h"

#include <cstring>
#include <new>

struct pypde_system {
  const pypde::SystemDesc *desc;
  pypde::SystemDesc *owned; // run-time compiled systems
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
  }
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

const char *pypde_last_error(void) { return last_error(); }

} // extern "C"
