/*
 * pypde_gb300.h -- C ABI of the GB300 ADER-WENO library
 * (pypde_gb300/libpypde_gb300.so).
 *
 * Drop-in for the C ABI of haranjackson/PyPDE (src/api.h), the boundary its
 * Python front end binds over ctypes (pypde/utils.py:9-16, 83-91).  All
 * buffers are the caller's host memory; the library copies them to the GPU,
 * runs every stage of the time step there and copies results back.  There
 * is no CPU fallback: without a usable GPU every entry point returns
 * PYPDE_ERR_CUDA.
 *
 * Callbacks.  The reference takes three host function pointers F, B, S
 * (numba cfuncs).  Device code cannot call host functions, so here F, B and
 * S are handles to one compiled device callback system (pypde_system): a
 * built-in system, or user source compiled at run time.  The ctypes
 * argument list is unchanged (three c_void_p), and each non-NULL handle
 * must name the same system.
 *
 * Return values: the reference's functions return void; these return a
 * status (PYPDE_OK = 0).  A ctypes binding with restype None ignores it.
 * pypde_last_error() gives a message for the last failure of this thread.
 */
#ifndef PYPDE_GB300_H
#define PYPDE_GB300_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PYPDE_OK 0
#define PYPDE_ERR_ARG 1         /* invalid argument or shape */
#define PYPDE_ERR_CUDA 2        /* CUDA error, or no GPU */
#define PYPDE_ERR_UNSUPPORTED 3 /* combination not built */
#define PYPDE_NAN_FOUND 4       /* NaN in the state; see pde_solver */
#define PYPDE_ERR_COMPILE 5     /* run-time compilation of callbacks failed */

typedef struct pypde_system pypde_system;
typedef struct pypde_warm_start pypde_warm_start;

/* Options and statistics of pde_solver_ex (extensions; no reference
 * counterpart).  Zero-initialise and set what you need. */
typedef struct {
  long long max_steps;   /* stop after this many steps; <= 0: run to tf */
  double newton_tol;     /* stiff form: ||obj||_inf tolerance; 0 -> 1e-12 */
  int device;            /* CUDA device ordinal */
  int steps_per_graph;   /* steps per CUDA graph launch; 0 -> automatic */
  int profile_stages;    /* 1: launch eagerly and time every stage with CUDA
                            events (fills pypde_stats.stage_seconds) */
  const pypde_warm_start *warm_start; /* stiff form: learned initial guess of
                            the Newton predictor (NULL: plain guess) */
  int mixed_precision;   /* stiff form: Newton sweeps in FP32 first, then at
                            least two FP64 sweeps to the same tolerance
                            (systems with FP32 callbacks only) */
  int strips;            /* the predictor runs in this many strips of cells,
                            the faces of finished strips on a second stream
                            meanwhile (results are identical for every
                            value); 0 -> automatic, 1 -> one launch each,
                            at most 32 */
} pypde_options;

/* Stages timed by pypde_options.profile_stages, in this order. */
#define PYPDE_STAGE_BOUNDARIES 0
#define PYPDE_STAGE_WENO 1
#define PYPDE_STAGE_CFL 2
#define PYPDE_STAGE_PREDICTOR 3
#define PYPDE_STAGE_FACES 4
#define PYPDE_STAGE_CENTERS 5
#define PYPDE_STAGE_GATHER 6
#define PYPDE_STAGE_OTHER 7
#define PYPDE_NSTAGES 8

typedef struct {
  long long steps;                 /* time steps taken */
  double t_final;                  /* time reached */
  unsigned long long pred_iters;   /* predictor iterations, summed over cells */
  int pred_max_iters;              /* largest per-cell iteration count */
  int pred_fail;                   /* cells whose Newton hit its cap */
  int nan_found;                   /* a NaN appeared in the state */
  double device_seconds;           /* time of the stepping loop on the GPU */
  long long kernel_launches;       /* kernels of this library launched */
  double stage_seconds[8];         /* per stage, with profile_stages */
  unsigned long long pred_fallbacks; /* warm-started cells that fell back to
                                      the plain guess */
  unsigned long long pred_iters32;   /* FP32 Newton sweeps, summed over cells */
} pypde_stats;

/* ---------------- callback systems ---------------- */

/* Built-in systems ("euler", "cattaneo", "ncp", "burgers2") for ndim 1-3.
 * No reference counterpart: stands in for pypde/cfuncs.py:30-75. */
int pypde_system_builtin(const char *name, int ndim, pypde_system **out);

/* Compile user callbacks given as CUDA C++ device code (see
 * pypde_gb300/callbacks.py, which translates Python F/B/S into this form).
 * src must define `struct UserSystem` with V, NDIM, HAS_F, HAS_B, HAS_S,
 * SECOND_ORDER and static __device__ F, B, S with the signatures of
 * pypde/cfuncs.py:6-8.  Stands in for pypde/cfuncs.py:30-75. */
int pypde_system_compile(const char *src, const char *name, int ndim, int V,
                         int has_F, int has_B, int has_S, int second_order,
                         pypde_system **out);

int pypde_system_info(const pypde_system *s, int *V, int *ndim, int *has_F,
                      int *has_B, int *has_S, int *second_order);
void pypde_system_free(pypde_system *s);

/* ---------------- the reference's entry points ---------------- */

/* Replaces pde_solver of src/api.h:4-10 / src/api.cpp:5-30.
 * u (in/out, prod(nX) x V) is advanced to tf, like the reference, which
 * writes the final state into the caller's array (api.cpp:18,
 * iterator.cpp:129).  ret (ndt x prod(nX) x V, caller-allocated) receives
 * the snapshots of iterator.cpp:136-150: row k when t first reaches
 * (k+1) tf / ndt, and row ndt-1 the final state.  STIFF selects the
 * locally implicit Newton predictor (else Picard, dg.cpp:187-202); FLUX
 * 0 Rusanov, 1 Roe, 2 Osher.  nThreads is accepted and ignored (one GPU).
 * On NaN the run stops; rows push and push+1 receive the last finite and
 * the first non-finite state (the reference writes them at
 * iterator.cpp:141-145 and keeps stepping) and PYPDE_NAN_FOUND is
 * returned. */
int pde_solver(const pypde_system *F, const pypde_system *B,
               const pypde_system *S, bool useF, bool useB, bool useS,
               double *u, double tf, int *nX, int ndim, double *dX, double CFL,
               int *boundaryTypes, bool STIFF, int FLUX, int N, int V, int ndt,
               bool secondOrder, double *ret, int nThreads);

/* pde_solver with options and statistics (extension). */
int pde_solver_ex(const pypde_system *sys, bool useF, bool useB, bool useS,
                  double *u, double tf, const int *nX, int ndim,
                  const double *dX, double CFL, const int *boundaryTypes,
                  bool STIFF, int FLUX, int N, int ndt, double *ret,
                  const pypde_options *opt, pypde_stats *stats);

/* Replaces weno_solver of src/api.h:12-13 / src/api.cpp:32-48: WENO
 * reconstruction of an already padded u (nX cells per axis) into ret,
 * shape (nX - 2(N-1)) x N^ndim x V. */
int weno_solver(double *ret, double *u, int *nX, int ndim, int N, int V);

/* weno_solver on caller-owned DEVICE buffers, for callers that cannot
 * allocate device memory (code running inside another framework's device
 * memory budget, or on paths where cudaMalloc's device synchronisation is
 * not allowed).  No counterpart in the reference.  u_dev (prod(nX) x V) and
 * ret_dev ((nX - 2(N-1)) x N^ndim x V) are device pointers; stream is a
 * cudaStream_t (NULL: the default stream); the call is asynchronous on it.
 * Allocates nothing: the passes between axes use one file-scope __device__
 * scratch array of 32 MiB (4 Mi doubles) that every GPU loading the library
 * holds until exit; larger grids are rejected with PYPDE_ERR_ARG.  All calls
 * share that array, so calls that overlap on the GPU (different streams,
 * other threads) race; serialise them.  The first call on a device looks up
 * the array's address (cudaGetSymbolAddress): make it before any stream
 * capture. */
int weno_solver_noalloc(double *ret_dev, const double *u_dev, const int *nX,
                        int ndim, int N, int V, void *stream);

/* ---------------- single stages (for checking each kernel) ------------ */

/* Ghost fill (src/grid/boundaries.cpp:25-53): u (prod nX x V) ->
 * ub (prod(nX+2N) x V). */
int pypde_boundaries(const double *u, const int *nX, int ndim,
                     const int *boundaryTypes, int N, int V, double *ub);

/* CFL timestep over the w-cells of w (TimeStepper::step,
 * src/solvers/stepper.cpp:35-76).  nrows = cells * N^ndim. */
int pypde_timestep(const pypde_system *sys, const double *w, long long nrows,
                   const double *dX, int ndim, int N, double CFL, double tf,
                   double t, long long count, double *dt_out);

/* Space-time predictor (DGSolver::predictor, src/solvers/dg/dg.cpp:204-224)
 * of every cell of w; qh gets N*nrows rows. */
int pypde_predictor(const pypde_system *sys, const double *w, long long nrows,
                    const double *dX, int ndim, int N, bool STIFF, double dt,
                    double newton_tol, double *qh, pypde_stats *stats);

/* Finite-volume corrector (FVSolver::apply, src/solvers/fv/fv.cpp:200-207):
 * u (prod nX x V) updated in place from qh over the (nX+2) grid. */
int pypde_fv(const pypde_system *sys, double *u, const double *qh,
             const int *nX, const double *dX, int ndim, int N, int FLUX,
             double dt);

/* Constant tables of order N, in the order nodes[N], wghts[N],
 * dervals[N*N], endvals[2N], dgmat[N*N], dgmat_inv[N*N], weno_inv[4][N*N],
 * sig[N*N] (4N + 8N^2 doubles).  Host-only; needs no GPU. */
int pypde_tables(int N, double *out);

/* FP64 FMA throughput of the device in TFLOP/s, measured by a dependent-
 * chain FMA loop: the roofline denominator of the FP64-bound kernels.
 * Bench support; no reference counterpart. */
int pypde_measure_fp64_peak(int device, double *tflops);

/* FP64 tensor-core (mma.sync m8n8k4 f64) throughput in TFLOP/s, measured by
 * independent chains of DMMA per warp: whether the predictor's small
 * contractions could gain from the tensor pipe.  Bench support; no
 * reference counterpart. */
int pypde_measure_dmma_peak(int device, double *tflops);

/* ---------------- batched problems (no reference counterpart) -----------
 * Many independent problems of one system (sizes, orders, boundary types
 * and end times may all differ) stepped together: every stage of a step is
 * one persistent launch per order whose CTAs drain a queue of cell tiles,
 * largest problems first, captured in a CUDA graph.  Each problem gives
 * the same bits as pde_solver_ex on it alone (ndt = 1: only the final
 * state is returned, written into u). */
typedef struct {
  double *u;             /* host, in/out, prod(nX) x V */
  double tf;
  int nX[3];             /* first ndim used */
  double dX[3];
  int boundaryTypes[3];  /* 0 transmissive, 1 periodic */
  int N;                 /* order */
  double cfl;
} pypde_problem;

typedef struct {
  long long max_steps;   /* per problem; <= 0: run to tf */
  double newton_tol;     /* stiff form; 0 -> 1e-12 */
  int device;
  int steps_per_graph;   /* 0 -> 8 */
  int autotune;          /* 1: the first five steps try, per stage, one block
                            per tile (0) and tiles-per-pop 1, 2, 4, 8 of the
                            persistent queue, and keep the fastest */
  int per_pop;           /* without autotune: tiles per queue pop, 0 = one
                            block per tile */
  int mixed_precision;   /* stiff form, built-in systems: FP32 Newton sweeps
                            first, as in pde_solver_ex */
  const pypde_warm_start *warm_start[4]; /* learned warm start of the
                            stiff predictor for the problems of order N
                            (index N = 1..3; NULL: plain guess), as in
                            pde_solver_ex; one batched guess launch per
                            order before its predictor */
} pypde_batch_options;

#define PYPDE_BATCH_STAGES 10 /* ghost, WENO x3, CFL, predictor, faces,
                                 centres, gather, warm-start guess */
typedef struct {
  long long steps;              /* summed over problems */
  long long max_problem_steps;
  double device_seconds;        /* the whole stepping loop, tuning included */
  long long kernel_launches;
  unsigned long long pred_iters;
  int nan_found;                /* problems stopped by a NaN */
  int per_pop[PYPDE_BATCH_STAGES]; /* tile shape chosen (first order group) */
  double tune_seconds;
} pypde_batch_stats;

/* steps_out, t_out: per-problem step counts and end times (may be NULL). */
int pde_solver_batch(const pypde_system *sys, bool STIFF, int FLUX, int nprob,
                     pypde_problem *problems, const pypde_batch_options *opt,
                     pypde_batch_stats *stats, long long *steps_out,
                     double *t_out);

/* ---------------- learned warm start (no reference counterpart) ---------
 * A per-cell MLP maps the WENO coefficients of a cell and log10(dt/tau) to
 * the initial guess of the stiff predictor's Newton iteration, which then
 * iterates to the same tolerance and falls back to the plain guess q = w
 * at the first iteration whose residual does not fall.  Network: feat
 * features padded to k1 -> 128 -> 128 -> no, SiLU, BF16 weights, FP32
 * accumulation.  Features of a cell: the V means over its N^ndim nodes,
 * the N^ndim*V deviations from them, log10(dt) - mean[tau_var] (log10(dt)
 * when tau_var < 0) and log10(r), all normalised by x_mean/x_scale, after
 * which the deviations are divided by their RMS r; outputs: the correction
 * qh - w at the N^(ndim+1)*V space-time values divided by r, padded to
 * no. */

/* Widths for (sys, N); PYPDE_ERR_UNSUPPORTED when sys has no source. */
int pypde_warm_start_shape(const pypde_system *sys, int N, int *feat, int *k1,
                           int *no);
/* Upload a trained network (FP32 host arrays; weights row-major [out][in]:
 * W1 128 x k1, W2 128 x 128, W3 no x 128; x = (f - x_mean) * x_scale;
 * correction = (y * y_scale + y_mean) * r). */
int pypde_warm_start_create(const pypde_system *sys, int N, int device,
                            const float *W1, const float *b1, const float *W2,
                            const float *b2, const float *W3, const float *b3,
                            const float *x_mean, const float *x_scale,
                            const float *y_mean, const float *y_scale,
                            int tau_var, pypde_warm_start **out);
int pypde_warm_start_free(pypde_warm_start *ws);

/* Stiff predictor started from an initial guess: the host array guess
 * (N*nrows x V) or, with guess NULL, the network warm. */
int pypde_predictor_guess(const pypde_system *sys, const double *w,
                          long long nrows, const double *dX, int ndim, int N,
                          double dt, double newton_tol, const double *guess,
                          const pypde_warm_start *warm, double *qh,
                          pypde_stats *stats);

/* Training pairs: runs pde_solver_ex for at most `steps` steps and, after
 * the predictor of step k, samples per_step reconstruction cells (every
 * stride-th, from an offset that changes with k): their WENO coefficients
 * (w_out, steps*per_step x N^ndim*V), converged predictor (qh_out,
 * steps*per_step x N^(ndim+1)*V) and dt (dt_out, steps). */
int pypde_harvest(const pypde_system *sys, double *u, double tf,
                  const int *nX, int ndim, const double *dX, double CFL,
                  const int *boundaryTypes, bool STIFF, int N, int steps,
                  long long per_step, long long stride, double *w_out,
                  double *qh_out, double *dt_out, const pypde_options *opt,
                  pypde_stats *stats);

/* Training kernels on device pointers, enqueued on `stream` (a
 * cudaStream_t; NULL = legacy default stream).
 * C[M][N] = sum_k A(m,k) B(k,n), A(m,k) = A[m*sam + k*sak],
 * B(k,n) = B[k*sbk + n*sbn], both rounded to BF16, FP32 accumulation;
 * then C += bias[n] and act = SiLU(C) when those pointers are non-NULL
 * (C may be NULL).  splits > 1 splits k, summed in a fixed order through
 * work (splits*M*N floats). */
int pypde_mlp_gemm(const float *A, long long sam, long long sak,
                   const float *B, long long sbk, long long sbn, float *C,
                   int M, int N, int K, int splits, float *work,
                   const float *bias, float *act, void *stream);
/* dZ = dA * SiLU'(Z), n elements. */
int pypde_mlp_silu_grad(const float *dA, const float *Z, float *dZ,
                        long long n, void *stream);
/* out[n] = sum over m of X[m][n] (M x N row-major), fixed order. */
int pypde_mlp_colsum(const float *X, int M, int N, float *out, void *stream);

const char *pypde_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
