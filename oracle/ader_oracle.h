/*
 * ader_oracle.h -- CPU restatement of PyPDE's ADER-WENO time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker, never the product: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * it.  The GPU library must not link, include or call anything here.
 *
 * Every function restates the algorithm of haranjackson/PyPDE src/ (paths
 * below are relative to that project) in plain C11 with row-major float64
 * arrays (the reference's Mat is row-major, src/types.h:21-22).  Parity of
 * this port with the reference itself is pinned by tests/golden/, whose
 * vectors are produced by the reference C++ compiled from its own sources
 * (oracle/Makefile target `ref`, driver oracle/ref_driver.cpp).
 */
#ifndef ADER_ORACLE_H
#define ADER_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Callback signatures of the reference (pypde/cfuncs.py:6-8, src/api.h:4-10) */
typedef void (*ora_flux_fn)(double *out, double *Q, double *dQ, int d);
typedef void (*ora_ncp_fn)(double *out, double *Q, int d);
typedef void (*ora_src_fn)(double *out, double *Q);
/* FP32 twins of the callbacks, for the FP32 Newton sweeps of the
 * mixed-precision stiff predictor (not in the reference). */
typedef void (*ora_flux32_fn)(float *out, const float *Q, const float *dQ, int d);
typedef void (*ora_ncp32_fn)(float *out, const float *Q, int d);
typedef void (*ora_src32_fn)(float *out, const float *Q);

#define ORA_MAXN 8
#define ORA_MAXV 24

/* Built-in test systems (oracle_systems.c).  Returns 0 on success. */
/* Active (transported) variables of a test system's flux in direction d:
 * their count (0 if the system declares none) and indices in idx. */
int ora_system_eig_active(ora_flux_fn F, int ndim, int d, int *idx);
int ora_system_lookup(const char *name, int ndim, int *V, ora_flux_fn *F,
                      ora_ncp_fn *B, ora_src_fn *S, int *secondOrder);
/* The FP32 callbacks of the same test system (null where it has none). */
int ora_system_lookup32(const char *name, int ndim, ora_flux32_fn *F,
                        ora_ncp32_fn *B, ora_src32_fn *S);

/* Constant tables of one (ndim, N) solver (src/poly/basis.cpp,
 * src/solvers/weno/weno_matrices.cpp, src/solvers/dg/dg_matrices.cpp). */
typedef struct {
  int N;
  double nodes[ORA_MAXN];             /* GL nodes on [0,1] */
  double wghts[ORA_MAXN];             /* GL weights on [0,1] */
  double dervals[ORA_MAXN * ORA_MAXN];/* DERVALS[i*N+j] = psi_j'(x_i) */
  double endvals[2 * ORA_MAXN];       /* ENDVALS[e*N+j] = psi_j(e) */
  double dgmat[ORA_MAXN * ORA_MAXN];  /* DG_MAT = psi psi^T(1) - <psi,psi'>^T */
  double dgmat_inv[ORA_MAXN * ORA_MAXN];
  double weno_inv[4][ORA_MAXN * ORA_MAXN]; /* inverses of mL, mR, mCL, mCR */
  double sig[ORA_MAXN * ORA_MAXN];    /* oscillation indicator matrix */
} ora_tables;

void ora_make_tables(int N, ora_tables *T);

/* Step stages.  Arrays are row-major (rows, V) float64. */
void ora_boundaries(const double *u, const int *nX, int ndim, const int *bt,
                    int N, int V, double *ub);
/* WENO reconstruction of an already padded array of shape nXb (weno_solver).
 * Output rows: prod(nXb - 2(N-1)) * N^ndim, each of V values. */
void ora_weno(const double *ub, const int *nXb, int ndim, int N, int V,
              double *w);
/* CFL timestep over nrows/Nd w-cells (TimeStepper::step). */
double ora_timestep(ora_flux_fn F, ora_ncp_fn B, const double *w, long nrows,
                    const double *dX, int ndim, int N, int V, double CFL,
                    double tf, double t, long count, int secondOrder);
/* Predictor over nrows/Nd w-cells; qh gets N*nrows rows.  Returns the total
 * number of Picard / Newton iterations; *maxit gets the per-cell maximum. */
long ora_predictor(ora_flux_fn F, ora_ncp_fn B, ora_src_fn S, const double *w,
                   long nrows, const double *dX, int ndim, int N, int V,
                   int stiff, double dt, double newton_tol, double *qh,
                   int *maxit, int secondOrder);
/* Stiff predictor started from a given guess (nrows/Nd cells x N Nd V,
 * e.g. a learned warm start), falling back per cell to the plain guess at
 * the first iteration whose residual does not fall; *fallbacks counts the
 * cells that fell back.  Not in the reference: the warm-start extension. */
long ora_predictor_guess(ora_flux_fn F, ora_ncp_fn B, ora_src_fn S,
                         const double *w, long nrows, const double *dX,
                         int ndim, int N, int V, double dt, double newton_tol,
                         const double *guess, double *qh, int *maxit,
                         long *fallbacks, int secondOrder);
/* The mixed-precision stiff predictor (not in the reference): per cell,
 * FP32 sweeps of the simplified Newton iteration with the FP32 callbacks
 * (at most 8; stopping at the FP32 rounding floor, at tol, when the
 * residual falls by less than half, or on a zero pivot), then the FP64
 * iteration from that iterate, which makes at least two updates before it
 * may stop at tol.  Returns the FP64 iterations; *sweeps32 (may be null)
 * gets the FP32 sweeps. */
long ora_predictor_mixed(ora_flux_fn F, ora_ncp_fn B, ora_src_fn S,
                         ora_flux32_fn F32, ora_ncp32_fn B32, ora_src32_fn S32,
                         const double *w, long nrows, const double *dX,
                         int ndim, int N, int V, double dt, double newton_tol,
                         double *qh, int *maxit, long *sweeps32,
                         int secondOrder);
/* The mixed form started from a given guess (the learned warm start with
 * FP32 sweeps): the FP32 sweeps start from the guess; the FP64 iteration
 * falls back to the plain guess as ora_predictor_guess does. */
long ora_predictor_guess_mixed(ora_flux_fn F, ora_ncp_fn B, ora_src_fn S,
                               ora_flux32_fn F32, ora_ncp32_fn B32,
                               ora_src32_fn S32, const double *w, long nrows,
                               const double *dX, int ndim, int N, int V,
                               double dt, double newton_tol,
                               const double *guess, double *qh, int *maxit,
                               long *fallbacks, long *sweeps32,
                               int secondOrder);
/* FV corrector (FVSolver::apply) on u (prod(nX) rows) using qh over the
 * w-grid nX+2. */
void ora_fv(ora_flux_fn F, ora_ncp_fn B, ora_src_fn S, double *u,
            const double *qh, const int *nX, const double *dX, int ndim,
            int N, int V, int flux, int secondOrder, double dt);

/* Whole solver (pde_solver, src/api.cpp:5-30 and src/solvers/iterator.cpp).
 * maxsteps < 0: run to tf.  Returns the number of steps taken; *t_out gets
 * the final time.  nThreads < 1 means "all host cores".  newton_tol is the
 * stiff residual tolerance (the reference uses 6e-6, dg.h:9). */
long ora_pde_solver(ora_flux_fn F, ora_ncp_fn B, ora_src_fn S, double *u,
                    double tf, const int *nX, int ndim, const double *dX,
                    double CFL, const int *bt, int stiff, int flux, int N,
                    int V, int ndt, int secondOrder, double *ret, int nThreads,
                    long maxsteps, double newton_tol, double *t_out);

/* ora_pde_solver with the mixed-precision stiff predictor (stiff implied). */
long ora_pde_solver_mixed(ora_flux_fn F, ora_ncp_fn B, ora_src_fn S,
                          ora_flux32_fn F32, ora_ncp32_fn B32, ora_src32_fn S32,
                          double *u, double tf, const int *nX, int ndim,
                          const double *dX, double CFL, const int *bt,
                          int flux, int N, int V, int ndt, int secondOrder,
                          double *ret, int nThreads, long maxsteps,
                          double newton_tol, double *t_out);

/* max |eigenvalue| of a general real n x n row-major matrix: FP32
 * eigenvalues refined in FP64 (ora_max_abs_eig), or the FP64 Francis QR
 * (ora_max_abs_eig_qr, destroys a). */
double ora_max_abs_eig(double *a, int n);
double ora_max_abs_eig_qr(double *a, int n);
/* Real eigen-decomposition: wr/wi eigenvalues, vr/vi eigenvectors (columns,
 * row-major n x n).  Returns 0 on success. */
int ora_eig(const double *a, int n, double *wr, double *wi, double *vr,
            double *vi);

#ifdef __cplusplus
}
#endif
#endif
