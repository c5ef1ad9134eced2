// kernels.cuh -- the ADER-WENO step as CUDA kernels for sm_103a.
//
// One step (src/solvers/iterator.cpp:99-148 of haranjackson/PyPDE):
//   k_boundaries      ghost fill u -> ub                 (a1)
//   k_weno_pass x d   reconstruction ub -> w             (a2)
//   k_cfl + k_dt      max|eig| reduction -> dt            (a3, a4)
//   k_predictor       space-time DG predictor w -> qh     (a5, a6)
//   k_faces           face fluxes (Rusanov, B path int.)  (a9, a10, a12)
//   k_centers         volume terms S - B grad q           (a8)
//   k_gather          u update in the reference's order   (a8, a9)
//   k_step_end        t, count, snapshot slot             (a14)
// Everything is FP64.  Data layout in HBM (row-major, V innermost, as the
// reference's Mat, src/types.h:21-22):
//   u  [C][V]                 C   = prod n_i
//   ub [Cb][V]                Cb  = prod (n_i + 2N)
//   w  [Cw][Nd][V]            Cw  = prod (n_i + 2), node index k_0 outermost
//   qh [Cw][N][Nd][V]         time node outermost inside a cell
//   face contributions [d][face][N][Nd_][2][V]
//   centre contributions [C][N][Nd][V]
// Device state (t, dt, count, flags) lives in a small struct in device
// memory so a whole run of steps can be captured in one CUDA graph; every
// kernel returns at once when the step is inactive (t >= tf or the step
// cap is reached).
#pragma once

#include "ader_common.cuh"
#include "eig_full.cuh"

namespace pypde {

// The block a kernel body works on: the hardware block of a one-problem
// launch, or one tile of one problem in a batched launch (b of n).
struct VBlock {
  long long b, n;
};

struct DevState {
  double t, dt, tf, cfl;
  double max_speed;  // CFL reduction target (non-negative doubles)
  long long count;   // steps taken
  long long max_steps;
  int active;        // current step runs
  int push;          // snapshots taken (ndt semantics)
  int snap_slot;     // ring slot written this step, or -1
  int nan_found;     // NaN seen in u after some step
  int nan_now;       // NaN seen in u after this step
  int ndt;
  unsigned long long pred_iters; // sum over cells of predictor iterations
  int pred_max_iters;
  int pred_fail;     // cells whose Newton iteration hit its cap
  unsigned long long pred_fallbacks; // warm-started cells reset to the plain guess
  unsigned long long pred_iters32;   // FP32 sweeps (mixed-precision form)
};

// Geometry of one problem, passed by value.
struct Geom {
  int ndim;
  int nX[3];  // interior cells
  int nXb[3]; // ghost-padded (n + 2N)
  int nXw[3]; // reconstruction grid (n + 2)
  int bt[3];  // 0 transmissive, 1 periodic
  double dX[3];
  long long C, Cb, Cw;
};

__device__ __forceinline__ bool step_active(const DevState *st) {
  return st->active != 0;
}

// ---------------------------------------------------------------------
// a1: ghost fill, grid/boundaries.cpp:7-53
// ---------------------------------------------------------------------
__device__ __forceinline__ int renorm_index(int ind, int N, int type,
                                            int bound) {
  int r = ind - N;
  if (r < 0)
    return type == 0 ? 0 : bound + r;
  if (r >= bound)
    return type == 0 ? bound - 1 : r - bound;
  return r;
}

// ---------------------------------------------------------------------
// a2: one WENO pass along axis d (weno.cpp:26-121).  in has shape
// m[0..ndim) x n4 nodes x V, out has m_d reduced by 2(N-1) and N*n4 nodes.
// One thread per (output cell, existing node, variable): the N nodal
// values of its 1-D reconstruction.
// ---------------------------------------------------------------------
template <int N>
__device__ __forceinline__ void k_weno_pass_body(VBlock vb_, const double *__restrict__ in,
                            double *__restrict__ out, long long n1, int md,
                            long long n3, int n4, int V, const Tables &T,
                            const DevState *st) {
  if (!step_active(st))
    return;
  constexpr int FN2 = (N - 1) / 2, CN2 = N / 2;
  constexpr int NST = (N > 2) ? ((N % 2 == 0) ? 4 : 3) : 2;
  const int n2 = md - 2 * (N - 1);
  long long total = n1 * n2 * n3 * (long long)n4 * V;
  for (long long e = vb_.b * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)vb_.n * blockDim.x) {
    long long r = e;
    int v = (int)(r % V);
    r /= V;
    int i4 = (int)(r % n4);
    r /= n4;
    long long i3 = r % n3;
    r /= n3;
    int i = (int)(r % n2);
    long long i1 = r / n2;
    const long long stride = n3 * n4 * (long long)V;
    const double *data =
        in + ((i1 * md + i) * n3 + i3) * n4 * (long long)V + i4 * V + v;
    double dat[2 * N - 1];
#pragma unroll
    for (int j = 0; j < 2 * N - 1; j++)
      dat[j] = data[j * stride];
    double num[N], den = 0;
#pragma unroll
    for (int k = 0; k < N; k++)
      num[k] = 0;
    const int starts[4] = {0, N - 1, FN2, CN2};
    const double lams[4] = {WENO_LAMS, WENO_LAMS, WENO_LAMC, WENO_LAMC};
#pragma unroll
    for (int k = 0; k < NST; k++) {
      double c[N];
#pragma unroll
      for (int a = 0; a < N; a++) {
        double s = 0;
#pragma unroll
        for (int j = 0; j < N; j++)
          s = fma(T.weno_inv[k][a * N + j], dat[starts[k] + j], s);
        c[a] = s;
      }
      double p = 0;
#pragma unroll
      for (int j = 0; j < N; j++) {
        double rr = 0;
#pragma unroll
        for (int a = 0; a < N; a++)
          rr = fma(c[a], T.sig[a * N + j], rr);
        p = fma(rr, c[j], p);
      }
      p += WENO_EPS;
      double p2 = p * p, p4 = p2 * p2, p8 = p4 * p4;
      double o = lams[k] / p8;
#pragma unroll
      for (int a = 0; a < N; a++)
        num[a] = fma(o, c[a], num[a]);
      den += o;
    }
    double *o = out + ((i1 * n2 + i) * n3 + i3) * (long long)n4 * N * V +
                (long long)i4 * N * V + v;
    const double rden = 1.0 / den;
#pragma unroll
    for (int a = 0; a < N; a++)
      o[a * V] = num[a] * rden;
  }
}

template <int N>
__global__ void k_weno_pass(const double *__restrict__ in,
                            double *__restrict__ out, long long n1, int md,
                            long long n3, int n4, int V, const __grid_constant__ Tables T,
                            const DevState *st) {
  k_weno_pass_body<N>(VBlock{(long long)blockIdx.x, (long long)gridDim.x}, in, out, n1, md, n3, n4, V, T, st);
}

// ---------------------------------------------------------------------
// a3/a4: CFL reduction, stepper.cpp:35-76.  One thread per w-cell.
// ---------------------------------------------------------------------
template <class Sys, int N>
__device__ __forceinline__ void k_cfl_body(VBlock vb_, const double *__restrict__ w, const Geom &g, const Tables &T,
          const double *__restrict__ wprod_g, DevState *st) {
  if (!step_active(st))
    return;
  constexpr int V = Sys::V, D = Sys::NDIM;
  constexpr int Nd = IPow<N, D>::value;
  __shared__ double wprod[Nd];
  __shared__ double dervals[N * N];
  for (int i = threadIdx.x; i < Nd; i += blockDim.x)
    wprod[i] = wprod_g[i];
  for (int i = threadIdx.x; i < N * N; i += blockDim.x)
    dervals[i] = T.dervals[i];
  __syncthreads();
  double local_max = 0.0;
  for (long long cell = vb_.b * (long long)blockDim.x + threadIdx.x;
       cell < g.Cw; cell += (long long)vb_.n * blockDim.x) {
    const double *w0 = w + cell * Nd * V;
    double q[V], dq[D * V];
    // q = WGHT_PRODS^T wh0 (stepper.cpp:49); wh0 starts cell Nd V doubles
    // into the reference's w buffer, with column stride V
    const bool rot = gemv_rot(V, V, cell * (long long)(Nd * V));
#pragma unroll
    for (int v = 0; v < V; v++)
      q[v] = gemv_lane(wprod, w0 + v, V, Nd, v < (V & ~1), rot);
#pragma unroll
    for (int d = 0; d < D; d++) {
      if (!Sys::SECOND_ORDER) { // F sees dQ only in the 2nd-order form
        for (int v = 0; v < V; v++)
          dq[d * V + v] = 0.0;
        continue;
      }
      int stride_d = 1;
      for (int e = d + 1; e < D; e++)
        stride_d *= N;
      // derivs (evaluations.cpp:23-47) as the reference rounds it: left to
      // right, each product and sum rounded, then divided by dX; dwh0 is a
      // buffer of its own there (stepper.cpp:38), so its average is aligned
      for (int v = 0; v < V; v++) {
        double dw[Nd];
        for (int idx = 0; idx < Nd; idx++) {
          int id = (idx / stride_d) % N;
          int base = idx - id * stride_d;
          double s = 0;
#pragma unroll
          for (int j = 0; j < N; j++)
            s = s + dervals[id * N + j] * w0[(base + j * stride_d) * V + v];
          dw[idx] = s / g.dX[d];
        }
        dq[d * V + v] = gemv_lane(wprod, dw, 1, Nd, v < (V & ~1), false);
      }
    }
    double tmp = 0.0;
#pragma unroll
    for (int d = 0; d < D; d++) {
      double lam = max_abs_eigs<Sys>(q, dq, d);
      if (Sys::SECOND_ORDER)
        lam += max_abs_eigs_2nd<Sys>(q, dq, d, N, g.dX[d]);
      tmp += lam / g.dX[d];
    }
    local_max = fmax(local_max, tmp);
  }
  // warp max, then one atomic per warp
  for (int off = 16; off > 0; off >>= 1)
    local_max = fmax(local_max, __shfl_down_sync(0xffffffffu, local_max, off));
  if ((threadIdx.x & 31) == 0)
    atomic_max_pos(&st->max_speed, local_max);
}

template <class Sys, int N>
__global__ void __launch_bounds__(128)
    k_cfl(const double *__restrict__ w, const __grid_constant__ Geom g, const __grid_constant__ Tables T,
          const double *__restrict__ wprod_g, DevState *st) {
  k_cfl_body<Sys, N>(VBlock{(long long)blockIdx.x, (long long)gridDim.x}, w, g, T, wprod_g, st);
}

// ---------------------------------------------------------------------
// a5/a6: space-time DG predictor, Picard form (dg.cpp:50-126, 156-224).
// A team of NT = N*Nd threads per cell, one per space-time node (t, idx);
// CPB cells per block.  Shared memory per cell: q0, r (NT x V) and the
// fluxes f (NT x D x V).
// ---------------------------------------------------------------------
template <class Sys, int N> struct PredCfg {
  static constexpr int V = Sys::V, D = Sys::NDIM;
  static constexpr int Nd = IPow<N, D>::value;
  static constexpr int NT = N * Nd;
  static constexpr int CPB_RAW = (NT >= 256) ? 1 : (256 / NT);
  static constexpr int CPB = CPB_RAW < 1 ? 1 : CPB_RAW;
  static constexpr int THREADS = CPB * NT;
  static constexpr int SMEM_DOUBLES = CPB * NT * V * (2 + D);
};

template <class Sys, int N>
__device__ __forceinline__ void k_predictor_body(VBlock vb_, const double *__restrict__ w,
                            double *__restrict__ qh, const Geom &g, const Tables &T,
                            const double *__restrict__ wprod_g,
                            DevState *st) {
  using Cfg = PredCfg<Sys, N>;
  constexpr int V = Cfg::V, D = Cfg::D, Nd = Cfg::Nd, NT = Cfg::NT;
  constexpr int CPB = Cfg::CPB;
  if (!step_active(st))
    return;
  const double dt = st->dt;
  extern __shared__ double smem[];
  double *s_q = smem;                    // [CPB][NT][V]
  double *s_r = s_q + CPB * NT * V;      // [CPB][NT][V]
  double *s_f = s_r + CPB * NT * V;      // [CPB][NT][D][V]
  __shared__ double wprod[Nd];
  __shared__ double dervals[N * N];
  __shared__ double dginv[N * N];
  __shared__ double wg[N];
  __shared__ int again[CPB];
  for (int i = threadIdx.x; i < Nd; i += blockDim.x)
    wprod[i] = wprod_g[i];
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) {
    dervals[i] = T.dervals[i];
    dginv[i] = T.dgmat_inv[i];
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x)
    wg[i] = T.wghts[i];

  const int lc = threadIdx.x / NT;   // local cell
  const int node = threadIdx.x % NT; // t * Nd + idx
  const int t = node / Nd, idx = node % Nd;
  const long long cell = (long long)vb_.b * CPB + lc;
  const bool valid = (lc < CPB) && (cell < g.Cw);
  int digs[D > 0 ? D : 1];
  {
    int rem = idx;
    for (int d = D - 1; d >= 0; d--) {
      digs[d] = rem % N;
      rem /= N;
    }
  }
  double *q0 = s_q + (lc * NT) * V;
  double *rr = s_r + (lc * NT) * V;
  double *ff = s_f + (lc * NT) * D * V;
  double Ww[V], q1[V];
  __syncthreads();
  if (valid) {
    // Ww[t,idx] = ENDVALS(0,t) prod W[i_d] w[idx]; q0[t,idx] = w[idx]
    // (dg.cpp:12-20, 156-171)
    double cc = T.endvals[t];
    for (int d = 0; d < D; d++)
      cc *= wg[digs[d]];
    const double *wc = w + (cell * Nd + idx) * V;
#pragma unroll
    for (int v = 0; v < V; v++) {
      double x = wc[v];
      Ww[v] = cc * x;
      q0[node * V + v] = x;
    }
  }
  bool done = !valid;
  int iters = 0;
  for (int it = 0; it < DG_IT; it++) {
    __syncthreads();
    double dq[D * V];
    if (!done) {
      // derivatives of q_t along each axis (evaluations.cpp:23-47); only
      // B and the second-order F read them
      if (Sys::SECOND_ORDER || Sys::HAS_B) {
#pragma unroll
        for (int d = 0; d < D; d++) {
          int sd = 1;
          for (int e = d + 1; e < D; e++)
            sd *= N;
          int base = idx - digs[d] * sd;
          const double rdx = 1.0 / g.dX[d];
#pragma unroll
          for (int v = 0; v < V; v++) {
            double s = 0;
#pragma unroll
            for (int j = 0; j < N; j++)
              s = fma(dervals[digs[d] * N + j],
                      q0[(t * Nd + base + j * sd) * V + v], s);
            dq[d * V + v] = s * rdx;
          }
        }
      }
      if (Sys::HAS_F) {
        // the node's state in registers: the parts of F shared by the D
        // directions (pressure, temperature, ...) are computed once
        double qr[V];
#pragma unroll
        for (int v = 0; v < V; v++)
          qr[v] = q0[node * V + v];
#pragma unroll
        for (int d = 0; d < D; d++)
          Sys::F(ff + (node * D + d) * V, qr, dq, d);
      }
    }
    __syncthreads();
    if (!done) {
      double r[V];
      if (Sys::HAS_S)
        Sys::S(r, q0 + node * V);
      else
#pragma unroll
        for (int v = 0; v < V; v++)
          r[v] = 0.0;
      double cc = wg[t];
#pragma unroll
      for (int d = 0; d < D; d++) {
        if (Sys::HAS_B) {
          double b[V * V];
          Sys::B(b, q0 + node * V, d);
#pragma unroll
          for (int i = 0; i < V; i++) {
            double acc = 0;
#pragma unroll
            for (int j = 0; j < V; j++)
              acc = fma(b[i * V + j], dq[d * V + j], acc);
            r[i] -= acc;
          }
        }
        if (Sys::HAS_F) {
          int sd = 1;
          for (int e = d + 1; e < D; e++)
            sd *= N;
          int base = idx - digs[d] * sd;
          const double rdx = 1.0 / g.dX[d];
#pragma unroll
          for (int v = 0; v < V; v++) {
            double s = 0;
#pragma unroll
            for (int j = 0; j < N; j++)
              s = fma(dervals[digs[d] * N + j],
                      ff[((t * Nd + base + j * sd) * D + d) * V + v], s);
            r[v] -= s * rdx;
          }
        }
        cc *= wg[digs[d]];
      }
#pragma unroll
      for (int v = 0; v < V; v++)
        rr[node * V + v] = r[v] * cc * dt + Ww[v]; // ret *= dt; ret += Ww
    }
    __syncthreads();
    if (lc < CPB && node == 0)
      again[lc] = 0;
    __syncthreads();
    if (!done) {
      // q1 = DG_U^{-1} r with DG_U = kron(DG_MAT, diag W, ...)
      bool more = false;
      const double rwp = 1.0 / wprod[idx];
#pragma unroll
      for (int v = 0; v < V; v++) {
        double s = 0;
#pragma unroll
        for (int k = 0; k < N; k++)
          s = fma(dginv[t * N + k], rr[(k * Nd + idx) * V + v], s);
        q1[v] = s * rwp;
        double a = q0[node * V + v];
        if (fabs(q1[v] - a) > DG_TOL * (1. + fabs(a)))
          more = true;
      }
      if (more)
        again[lc] = 1;
    }
    __syncthreads();
    if (!done) {
      iters = it + 1;
      if (again[lc]) {
#pragma unroll
        for (int v = 0; v < V; v++)
          q0[node * V + v] = q1[v];
      } else {
        done = true;
      }
    }
    if (__syncthreads_and(done))
      break;
  }
  if (valid) {
    double *o = qh + (cell * NT + node) * V;
#pragma unroll
    for (int v = 0; v < V; v++)
      o[v] = q1[v];
    if (node == 0) {
      atomicAdd(&st->pred_iters, (unsigned long long)iters);
      atomicMax(&st->pred_max_iters, iters);
    }
  }
}

template <class Sys, int N>
__global__ void k_predictor(const double *__restrict__ w,
                            double *__restrict__ qh, const __grid_constant__ Geom g, const __grid_constant__ Tables T,
                            const double *__restrict__ wprod_g,
                            DevState *st, long long b0) {
  // b0: first block of a strip of cells (0 for the whole grid)
  k_predictor_body<Sys, N>(VBlock{b0 + blockIdx.x, b0 + gridDim.x}, w, qh, g, T, wprod_g, st);
}

// ---------------------------------------------------------------------
// a7: stiff predictor.  Locally implicit Newton iteration on
// obj(q) = rhs(q) - DG_U q (dg.cpp:128-154): the source is linearised
// exactly at every space-time node, the fluxes are kept explicit.  Per
// spatial node idx the (N V) x (N V) system
//   A[(t,v),(k,w)] = dt W_t dS_v/dq_w(q_t) [t = k] - DG_MAT[t,k] [v = w]
// is factored (LU, partial pivoting) and q <- q - A^{-1} obj(q) / prod W_idx.
// Stops at ||obj||_inf <= tol, or at the rounding floor of obj
// (16 eps max(|rhs|, |DG_U q|)).  Same operation order as the host
// restatement's dg_newton.  Replaces the reference's Newton-Krylov
// (dg.cpp:173-185, scipy/algos/newton_krylov.cpp), whose absolute
// tolerance is 6e-6, by an iteration to tol (default 1e-12).
//
// With guess != 0 the iteration starts from the values already in qh (a
// learned warm start) instead of the plain guess q = w.  A cell whose
// residual does not fall below the previous iteration's, or has an entry
// that is not finite, spends that iteration resetting q to the plain guess
// and then runs the plain iteration; pred_fallbacks counts those cells.
// ---------------------------------------------------------------------
constexpr int NEWTON_MAXIT = 200;

template <class Sys, int N> struct NewtonCfg {
  static constexpr int V = Sys::V, D = Sys::NDIM;
  static constexpr int Nd = IPow<N, D>::value;
  static constexpr int NT = N * Nd;
  static constexpr int NL = N * V; // size of one spatial node's system
  static constexpr int CELL_DOUBLES = NT * V * (2 + D) + Nd * NL * NL;
  static constexpr int CELL_BYTES = CELL_DOUBLES * 8 + Nd * NL * 4;
  static constexpr int BY_THREADS = (NT >= 128) ? 1 : 128 / NT;
  static constexpr int BY_SMEM = (100 * 1024) / CELL_BYTES;
  static constexpr int CPB_RAW = BY_THREADS < BY_SMEM ? BY_THREADS : BY_SMEM;
  static constexpr int CPB = CPB_RAW < 1 ? 1 : CPB_RAW;
  static constexpr int THREADS = CPB * NT;
  static constexpr size_t SMEM_BYTES = (size_t)CPB * CELL_BYTES;
};

// FP32 sweeps of the mixed-precision stiff predictor: the simplified
// Newton iteration of k_newton with every quantity in FP32 -- callbacks
// instantiated with float, the FD step sqrt(eps_32) max(|q|, 1), the LU in
// FP32 and built once -- started from the cell's q and written back into
// it.  A cell stops at its FP32 rounding floor (residual <= 64 eps_32
// scale), at tol, when the residual falls by less than half in a sweep, on
// a zero pivot, or after NEWTON32_MAXIT sweeps.  Shared scratch: q32 and r32
// in s_r, fluxes in s_f, the LU in s_A (the FP64 loop rebuilds all three).
// Returns this thread's cell's sweep count.
constexpr int NEWTON32_MAXIT = 8;

template <class Sys, int N>
__device__ __forceinline__ int newton_fp32_sweeps(
    double *s_q, double *s_r, double *s_f, double *s_A, int *s_piv,
    const double *Ww, const double *wprod, const double *dervals,
    const double *dgmat, const double *wg, const Geom &g, double dt,
    double tol, int lc, int node, int t, int idx, const int *digs,
    bool valid) {
  using Cfg = NewtonCfg<Sys, N>;
  constexpr int V = Cfg::V, D = Cfg::D, Nd = Cfg::Nd, NT = Cfg::NT;
  constexpr int NL = Cfg::NL, CPB = Cfg::CPB;
  constexpr float EPS32 = 1.1920928955078125e-07f;
  constexpr float SQRT_EPS32 = 3.4526698300124393e-04f;
  __shared__ float wprod32[Nd], dervals32[N * N], dgmat32[N * N], wg32[N];
  __shared__ unsigned int res32[CPB], scale32[CPB];
  __shared__ int done32[CPB], lu32[CPB];
  __shared__ float last32[CPB];
  for (int i = threadIdx.x; i < Nd; i += blockDim.x)
    wprod32[i] = (float)wprod[i];
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) {
    dervals32[i] = (float)dervals[i];
    dgmat32[i] = (float)dgmat[i];
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x)
    wg32[i] = (float)wg[i];
  float *q32 = (float *)s_r + (lc * NT) * V;
  float *f32 = (float *)s_f + (lc * NT) * D * V;
  float *r32 = (float *)s_r + CPB * NT * V + (lc * NT) * V;
  float *A32 = (float *)s_A + (lc * Nd + idx) * NL * NL;
  int *piv = s_piv + (lc * Nd + idx) * NL;
  float Ww32[V];
  if (threadIdx.x < CPB) {
    done32[threadIdx.x] = 0;
    lu32[threadIdx.x] = 0;
    last32[threadIdx.x] = 3.0e38f;
  }
  if (valid) {
#pragma unroll
    for (int v = 0; v < V; v++) {
      q32[node * V + v] = (float)s_q[(lc * NT + node) * V + v];
      Ww32[v] = (float)Ww[v];
    }
  } else if (lc < CPB && node == 0) {
    done32[lc] = 1;
  }
  const float dt32 = (float)dt, tol32 = (float)tol;
  int sweeps = 0;
  for (int it = 0; it < NEWTON32_MAXIT; it++) {
    if (lc < CPB && node == 0) {
      res32[lc] = 0u;
      scale32[lc] = 0u;
    }
    __syncthreads();
    const bool active = valid && !done32[lc];
    float dq[D * V];
    if (active) {
      if (Sys::SECOND_ORDER || Sys::HAS_B) {
#pragma unroll
        for (int d = 0; d < D; d++) {
          int sd = 1;
          for (int e = d + 1; e < D; e++)
            sd *= N;
          const int base = idx - digs[d] * sd;
          const float rdx = 1.0f / (float)g.dX[d];
#pragma unroll
          for (int v = 0; v < V; v++) {
            float sacc = 0.0f;
#pragma unroll
            for (int j = 0; j < N; j++)
              sacc = fmaf(dervals32[digs[d] * N + j],
                          q32[(t * Nd + base + j * sd) * V + v], sacc);
            dq[d * V + v] = sacc * rdx;
          }
        }
      }
      if (Sys::HAS_F) {
        float qr[V];
#pragma unroll
        for (int v = 0; v < V; v++)
          qr[v] = q32[node * V + v];
#pragma unroll
        for (int d = 0; d < D; d++)
          Sys::F(f32 + (node * D + d) * V, qr, dq, d);
      }
    }
    __syncthreads();
    if (active) {
      float r[V];
      if (Sys::HAS_S)
        Sys::S(r, q32 + node * V);
      else
#pragma unroll
        for (int v = 0; v < V; v++)
          r[v] = 0.0f;
      float cc = wg32[t];
#pragma unroll
      for (int d = 0; d < D; d++) {
        if (Sys::HAS_B) {
          float b[V * V];
          Sys::B(b, q32 + node * V, d);
#pragma unroll
          for (int i = 0; i < V; i++) {
            float acc = 0.0f;
#pragma unroll
            for (int j = 0; j < V; j++)
              acc = fmaf(b[i * V + j], dq[d * V + j], acc);
            r[i] -= acc;
          }
        }
        if (Sys::HAS_F) {
          int sd = 1;
          for (int e = d + 1; e < D; e++)
            sd *= N;
          const int base = idx - digs[d] * sd;
          const float rdx = 1.0f / (float)g.dX[d];
#pragma unroll
          for (int v = 0; v < V; v++) {
            float sacc = 0.0f;
#pragma unroll
            for (int j = 0; j < N; j++)
              sacc = fmaf(dervals32[digs[d] * N + j],
                          f32[((t * Nd + base + j * sd) * D + d) * V + v], sacc);
            r[v] -= sacc * rdx;
          }
        }
        cc *= wg32[digs[d]];
      }
      unsigned int rm = 0u, sm = 0u;
#pragma unroll
      for (int v = 0; v < V; v++) {
        const float rv = fmaf(r[v] * cc, dt32, Ww32[v]);
        float uq = 0.0f;
#pragma unroll
        for (int k = 0; k < N; k++)
          uq = fmaf(dgmat32[t * N + k], q32[(k * Nd + idx) * V + v], uq);
        uq *= wprod32[idx];
        const float ov = rv - uq;
        r32[node * V + v] = ov;
        const unsigned int a = __float_as_uint(ov) & 0x7fffffffu;
        const unsigned int b = __float_as_uint(rv) & 0x7fffffffu;
        const unsigned int c = __float_as_uint(uq) & 0x7fffffffu;
        // a NaN or infinity stops the cell's FP32 sweeps (the max is the
        // largest finite bit pattern then)
        rm = max(rm, a >= 0x7f800000u ? 0x7f7fffffu : a);
        sm = max(sm, max(b < 0x7f800000u ? b : 0u, c < 0x7f800000u ? c : 0u));
      }
      atomicMax(&res32[lc], rm);
      atomicMax(&scale32[lc], sm);
    }
    __syncthreads();
    bool stop = false;
    if (active) {
      const float res = __uint_as_float(res32[lc]);
      const float scale = __uint_as_float(scale32[lc]);
      stop = res <= tol32 || res <= 64.0f * EPS32 * scale ||
             !(res <= 0.5f * last32[lc]) || res >= 3.0e38f;
      if (!stop && !lu32[lc]) {
        // row block t of A: the FD Jacobian of S in FP32
        float qn[V], s0[V], s1[V];
#pragma unroll
        for (int v = 0; v < V; v++)
          qn[v] = q32[node * V + v];
        if (Sys::HAS_S)
          Sys::S(s0, qn);
#pragma unroll
        for (int wv = 0; wv < V; wv++) {
          float ih = 0.0f;
          if (Sys::HAS_S) {
            const float q0 = qn[wv];
            const float h = fmaxf(SQRT_EPS32 * fabsf(q0), SQRT_EPS32);
            qn[wv] = q0 + h;
            Sys::S(s1, qn);
            qn[wv] = q0;
            ih = 1.0f / h;
          }
          for (int v = 0; v < V; v++)
            for (int k = 0; k < N; k++) {
              float a = 0.0f;
              if (k == t && Sys::HAS_S)
                a = dt32 * wg32[t] * ((s1[v] - s0[v]) * ih);
              A32[(t * V + v) * NL + k * V + wv] = a;
            }
        }
        for (int k = 0; k < N; k++)
          for (int v = 0; v < V; v++)
            A32[(t * V + v) * NL + k * V + v] -= dgmat32[t * N + k];
      }
    }
    __syncthreads();
    bool bad = false;
    if (active && !stop && t == 0) {
      bool ok = true;
      for (int k = 0; k < NL && ok && !lu32[lc]; k++) {
        int p = k;
        unsigned int pm = __float_as_uint(A32[k * NL + k]) & 0x7fffffffu;
        for (int i = k + 1; i < NL; i++) {
          const unsigned int m = __float_as_uint(A32[i * NL + k]) & 0x7fffffffu;
          if (m > pm) {
            p = i;
            pm = m;
          }
        }
        piv[k] = p;
        if (pm == 0u) {
          ok = false;
          break;
        }
        if (p != k)
          for (int j = 0; j < NL; j++) {
            const float tmp = A32[k * NL + j];
            A32[k * NL + j] = A32[p * NL + j];
            A32[p * NL + j] = tmp;
          }
        const float rp = 1.0f / A32[k * NL + k];
        for (int i = k + 1; i < NL; i++) {
          const float f = A32[i * NL + k] * rp;
          A32[i * NL + k] = f;
          if ((__float_as_uint(f) & 0x7fffffffu) == 0u)
            continue;
          for (int j = k + 1; j < NL; j++)
            A32[i * NL + j] = fmaf(-f, A32[k * NL + j], A32[i * NL + j]);
        }
      }
      if (!ok) {
        bad = true;
      } else {
        float b[NL];
        const float rwp = 1.0f / wprod32[idx];
        for (int tt = 0; tt < N; tt++)
          for (int v = 0; v < V; v++)
            b[tt * V + v] = r32[(tt * Nd + idx) * V + v] * rwp;
        for (int k = 0; k < NL; k++)
          if (piv[k] != k) {
            const float tmp = b[k];
            b[k] = b[piv[k]];
            b[piv[k]] = tmp;
          }
        for (int k = 0; k < NL; k++)
          for (int i = k + 1; i < NL; i++)
            if ((__float_as_uint(A32[i * NL + k]) & 0x7fffffffu) != 0u)
              b[i] = fmaf(-A32[i * NL + k], b[k], b[i]);
        for (int i = NL - 1; i >= 0; i--) {
          float sacc = b[i];
          for (int j = i + 1; j < NL; j++)
            if ((__float_as_uint(A32[i * NL + j]) & 0x7fffffffu) != 0u)
              sacc = fmaf(-A32[i * NL + j], b[j], sacc);
          b[i] = sacc / A32[i * NL + i];
        }
        for (int tt = 0; tt < N; tt++)
          for (int v = 0; v < V; v++)
            q32[(tt * Nd + idx) * V + v] -= b[tt * V + v];
      }
    }
    if (bad)
      atomicOr(&done32[lc], 2);
    __syncthreads();
    if (active && node == 0) {
      if (stop) {
        done32[lc] |= 1;
      } else {
        last32[lc] = __uint_as_float(res32[lc]);
        lu32[lc] = 1;
        sweeps = it + 1;
      }
    }
    bool all_done = true;
    if (node == 0 && lc < CPB)
      all_done = done32[lc] != 0;
    if (__syncthreads_and(all_done))
      break;
  }
  // hand the FP32 iterate to the FP64 sweeps
  if (valid) {
#pragma unroll
    for (int v = 0; v < V; v++)
      s_q[(lc * NT + node) * V + v] = (double)q32[node * V + v];
  }
  __syncthreads();
  return sweeps;
}

template <class Sys, int N>
__device__ __forceinline__ void k_newton_body(VBlock vb_, const double *__restrict__ w, double *__restrict__ qh,
                         const Geom &g, const Tables &T, const double *__restrict__ wprod_g,
                         DevState *st, double tol, int guess, int mixed) {
  using Cfg = NewtonCfg<Sys, N>;
  constexpr int V = Cfg::V, D = Cfg::D, Nd = Cfg::Nd, NT = Cfg::NT;
  constexpr int NL = Cfg::NL, CPB = Cfg::CPB;
  if (!step_active(st))
    return;
  const double dt = st->dt;
  extern __shared__ double smem[];
  double *s_q = smem;                        // [CPB][NT][V]
  double *s_r = s_q + CPB * NT * V;          // [CPB][NT][V]
  double *s_f = s_r + CPB * NT * V;          // [CPB][NT][D][V]
  double *s_A = s_f + CPB * NT * D * V;      // [CPB][Nd][NL][NL]
  int *s_piv = (int *)(s_A + CPB * Nd * NL * NL); // [CPB][Nd][NL]
  __shared__ double wprod[Nd];
  __shared__ double dervals[N * N];
  __shared__ double dgmat[N * N];
  __shared__ double wg[N];
  __shared__ unsigned long long res_bits[CPB], scale_bits[CPB];
  __shared__ int cell_done[CPB];
  __shared__ int on_guess[CPB], bad_res[CPB], have_lu[CPB];
  __shared__ double prev_res[CPB], last_res[CPB];
  for (int i = threadIdx.x; i < Nd; i += blockDim.x)
    wprod[i] = wprod_g[i];
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) {
    dervals[i] = T.dervals[i];
    dgmat[i] = T.dgmat[i];
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x)
    wg[i] = T.wghts[i];

  const int lc = threadIdx.x / NT;
  const int node = threadIdx.x % NT;
  const int t = node / Nd, idx = node % Nd;
  const long long cell = (long long)vb_.b * CPB + lc;
  const bool valid = (lc < CPB) && (cell < g.Cw);
  int digs[D > 0 ? D : 1];
  {
    int rem = idx;
    for (int d = D - 1; d >= 0; d--) {
      digs[d] = rem % N;
      rem /= N;
    }
  }
  double *q = s_q + (lc * NT) * V;
  double *rr = s_r + (lc * NT) * V;
  double *ff = s_f + (lc * NT) * D * V;
  double Ww[V];
  if (threadIdx.x < CPB) {
    cell_done[threadIdx.x] = 0;
    on_guess[threadIdx.x] = guess != 0;
    prev_res[threadIdx.x] = __longlong_as_double(0x7ff0000000000000LL); // +inf
    last_res[threadIdx.x] = __longlong_as_double(0x7ff0000000000000LL);
    have_lu[threadIdx.x] = 0;
  }
  __syncthreads();
  const double *wc = w + (cell * Nd + idx) * V;
  if (valid) {
    double cc = T.endvals[t];
    for (int d = 0; d < D; d++)
      cc *= wg[digs[d]];
    const double *gq = qh + (cell * NT + node) * V;
#pragma unroll
    for (int v = 0; v < V; v++) {
      double x = wc[v];
      Ww[v] = cc * x;
      q[node * V + v] = guess ? gq[v] : x;
    }
  } else if (lc < CPB && node == 0) {
    cell_done[lc] = 1;
  }
  if constexpr (Sys::HAS_FP32) {
    if (mixed) {
      __syncthreads();
      const int sw = newton_fp32_sweeps<Sys, N>(
          s_q, s_r, s_f, s_A, s_piv, Ww, wprod, dervals, dgmat, wg, g, dt,
          tol, lc, node, t, idx, digs, valid);
      if (valid && node == 0)
        atomicAdd(&st->pred_iters32, (unsigned long long)sw);
    }
  }
  // mixed precision: at least two FP64 updates before a cell may stop
  const int min_updates = mixed ? 2 : 0;
  int iters = 0;
  bool failed = false;
  for (int it = 0; it < NEWTON_MAXIT; it++) {
    if (lc < CPB && node == 0) {
      res_bits[lc] = 0ULL;
      scale_bits[lc] = 0ULL;
      bad_res[lc] = 0;
    }
    __syncthreads();
    const bool active = valid && !cell_done[lc];
    double dq[D * V];
    if (active) {
      if (Sys::SECOND_ORDER || Sys::HAS_B) {
#pragma unroll
        for (int d = 0; d < D; d++) {
          int sd = 1;
          for (int e = d + 1; e < D; e++)
            sd *= N;
          int base = idx - digs[d] * sd;
          const double rdx = 1.0 / g.dX[d];
#pragma unroll
          for (int v = 0; v < V; v++) {
            double s = 0;
#pragma unroll
            for (int j = 0; j < N; j++)
              s = fma(dervals[digs[d] * N + j],
                      q[(t * Nd + base + j * sd) * V + v], s);
            dq[d * V + v] = s * rdx;
          }
        }
      }
      if (Sys::HAS_F) {
        // the node's state in registers: the parts of F shared by the D
        // directions (pressure, temperature, ...) are computed once
        double qr[V];
#pragma unroll
        for (int v = 0; v < V; v++)
          qr[v] = q[node * V + v];
#pragma unroll
        for (int d = 0; d < D; d++)
          Sys::F(ff + (node * D + d) * V, qr, dq, d);
      }
    }
    __syncthreads();
    if (active) {
      double r[V];
      if (Sys::HAS_S)
        Sys::S(r, q + node * V);
      else
#pragma unroll
        for (int v = 0; v < V; v++)
          r[v] = 0.0;
      double cc = wg[t];
#pragma unroll
      for (int d = 0; d < D; d++) {
        if (Sys::HAS_B) {
          double b[V * V];
          Sys::B(b, q + node * V, d);
#pragma unroll
          for (int i = 0; i < V; i++) {
            double acc = 0;
#pragma unroll
            for (int j = 0; j < V; j++)
              acc = fma(b[i * V + j], dq[d * V + j], acc);
            r[i] -= acc;
          }
        }
        if (Sys::HAS_F) {
          int sd = 1;
          for (int e = d + 1; e < D; e++)
            sd *= N;
          int base = idx - digs[d] * sd;
          const double rdx = 1.0 / g.dX[d];
#pragma unroll
          for (int v = 0; v < V; v++) {
            double s = 0;
#pragma unroll
            for (int j = 0; j < N; j++)
              s = fma(dervals[digs[d] * N + j],
                      ff[((t * Nd + base + j * sd) * D + d) * V + v], s);
            r[v] -= s * rdx;
          }
        }
        cc *= wg[digs[d]];
      }
      // max |.| over the entries that are not NaN, as integer maxima of
      // the magnitude bits (the ordering of non-negative doubles)
      unsigned long long res = 0, scale = 0;
      bool bad = false;
#pragma unroll
      for (int v = 0; v < V; v++) {
        double rv = r[v] * cc * dt + Ww[v]; // ret *= dt; ret += Ww
        double uq = 0;
#pragma unroll
        for (int k = 0; k < N; k++)
          uq = fma(dgmat[t * N + k], q[(k * Nd + idx) * V + v], uq);
        uq *= wprod[idx];
        double ov = rv - uq;
        rr[node * V + v] = ov;
        const unsigned long long a = mag_bits(ov), b = mag_bits(rv),
                                 c2 = mag_bits(uq);
        if (a <= INF_BITS && a > res)
          res = a;
        if (b <= INF_BITS && b > scale)
          scale = b;
        if (c2 <= INF_BITS && c2 > scale)
          scale = c2;
        bad |= a >= INF_BITS;
      }
      if (bad)
        bad_res[lc] = 1;
      atomicMax(&res_bits[lc], res);
      atomicMax(&scale_bits[lc], scale);
    }
    __syncthreads();
    bool conv = false, reset = false, refresh = false;
    double res = 0.0;
    if (active) {
      res = __longlong_as_double((long long)res_bits[lc]);
      double scale = __longlong_as_double((long long)scale_bits[lc]);
      reset = on_guess[lc] && (bad_res[lc] || !(res < prev_res[lc]));
      conv = !reset && it >= min_updates &&
             (res <= tol || res <= 16 * DBL_EPS * scale);
      // simplified Newton: factors reused until the residual falls by
      // less than half in an iteration
      refresh = !have_lu[lc] || !(res <= 0.5 * last_res[lc]);
      if (reset) {
#pragma unroll
        for (int v = 0; v < V; v++)
          q[node * V + v] = wc[v];
      } else if (!conv && refresh) {
        // row block t of A for spatial node idx: the FD Jacobian of S
        double *A = s_A + ((lc * Nd) + idx) * NL * NL;
        // the node's state in registers and the column loop unrolled: each
        // column's perturbed variable is a constant, so the parts of S that
        // do not depend on it are computed once
        double qn[V], s0[V], s1[V];
#pragma unroll
        for (int v = 0; v < V; v++)
          qn[v] = q[node * V + v];
        if (Sys::HAS_S)
          Sys::S(s0, qn);
#pragma unroll
        for (int wv = 0; wv < V; wv++) {
          double ih = 0.0;
          if (Sys::HAS_S) {
            double q0 = qn[wv], h;
            fd_step_pow2(q0, h, ih);
            qn[wv] = q0 + h;
            Sys::S(s1, qn);
            qn[wv] = q0;
          }
          for (int v = 0; v < V; v++)
            for (int k = 0; k < N; k++) {
              double a = 0.0;
              if (k == t && Sys::HAS_S)
                a = dt * wg[t] * ((s1[v] - s0[v]) * ih);
              A[(t * V + v) * NL + k * V + wv] = a;
            }
        }
        for (int k = 0; k < N; k++)
          for (int v = 0; v < V; v++)
            A[(t * V + v) * NL + k * V + v] -= dgmat[t * N + k];
      }
    }
    __syncthreads();
    if (active && !conv && !reset && t == 0) {
      // LU with partial pivoting of A (when refreshed), then solve for the
      // update of node idx at every time node (lu_factor / lu_solve of the
      // restatement).  Magnitude comparisons and zero tests are done on
      // the bits: the same decisions for every value that is not NaN.
      double *A = s_A + ((lc * Nd) + idx) * NL * NL;
      int *piv = s_piv + ((lc * Nd) + idx) * NL;
      bool ok = true;
      for (int k = 0; k < NL && ok && refresh; k++) {
        int p = k;
        unsigned long long pm = mag_bits(A[k * NL + k]);
        for (int i = k + 1; i < NL; i++) {
          const unsigned long long m = mag_bits(A[i * NL + k]);
          if (m > pm) {
            p = i;
            pm = m;
          }
        }
        piv[k] = p;
        if (pm == 0ULL) {
          ok = false;
          break;
        }
        if (p != k)
          for (int j = 0; j < NL; j++) {
            double tmp = A[k * NL + j];
            A[k * NL + j] = A[p * NL + j];
            A[p * NL + j] = tmp;
          }
        const double rp = 1.0 / A[k * NL + k];
        for (int i = k + 1; i < NL; i++) {
          double f = A[i * NL + k] * rp;
          A[i * NL + k] = f;
          if (mag_bits(f) == 0ULL) // structural zero: the row is unchanged
            continue;
          for (int j = k + 1; j < NL; j++)
            A[i * NL + j] = fma(-f, A[k * NL + j], A[i * NL + j]);
        }
        A[k * NL + k] = rp; // U's diagonal kept as reciprocals for the solves
      }
      if (!ok) {
        failed = true;
      } else {
        double b[NL];
        const double rw = 1.0 / wprod[idx];
        for (int tt = 0; tt < N; tt++)
          for (int v = 0; v < V; v++)
            b[tt * V + v] = rr[(tt * Nd + idx) * V + v] * rw;
        // rows were swapped whole (L included): permute b first
        for (int k = 0; k < NL; k++)
          if (piv[k] != k) {
            double tmp = b[k];
            b[k] = b[piv[k]];
            b[piv[k]] = tmp;
          }
        for (int k = 0; k < NL; k++)
          for (int i = k + 1; i < NL; i++)
            if (mag_bits(A[i * NL + k]) != 0ULL)
              b[i] = fma(-A[i * NL + k], b[k], b[i]);
        for (int i = NL - 1; i >= 0; i--) {
          double sacc = b[i];
          for (int j = i + 1; j < NL; j++)
            if (mag_bits(A[i * NL + j]) != 0ULL)
              sacc = fma(-A[i * NL + j], b[j], sacc);
          b[i] = sacc * A[i * NL + i]; // the pivot's reciprocal
        }
        for (int tt = 0; tt < N; tt++)
          for (int v = 0; v < V; v++)
            q[(tt * Nd + idx) * V + v] -= b[tt * V + v];
      }
    }
    if (failed)
      atomicOr(&cell_done[lc], 2);
    __syncthreads();
    if (active && node == 0) {
      if (reset) {
        on_guess[lc] = 0;
        have_lu[lc] = 0;
        last_res[lc] = __longlong_as_double(0x7ff0000000000000LL);
        atomicAdd(&st->pred_fallbacks, 1ULL);
      } else {
        if (on_guess[lc])
          prev_res[lc] = res;
        if (!conv) {
          last_res[lc] = res;
          if (refresh)
            have_lu[lc] = 1;
        }
      }
      if (conv)
        cell_done[lc] |= 1;
      else
        iters = it + 1;
    }
    if (active && conv && node == 0)
      iters = it;
    bool all_done = true;
    if (node == 0 && lc < CPB)
      all_done = cell_done[lc] != 0;
    if (__syncthreads_and(all_done))
      break;
  }
  if (valid) {
    double *o = qh + (cell * NT + node) * V;
#pragma unroll
    for (int v = 0; v < V; v++)
      o[v] = q[node * V + v];
    if (node == 0) {
      atomicAdd(&st->pred_iters, (unsigned long long)iters);
      atomicMax(&st->pred_max_iters, iters);
      if (cell_done[lc] != 1)
        atomicAdd(&st->pred_fail, 1);
    }
  }
}

template <class Sys, int N>
__global__ void k_newton(const double *__restrict__ w, double *__restrict__ qh,
                         const __grid_constant__ Geom g, const __grid_constant__ Tables T, const double *__restrict__ wprod_g,
                         DevState *st, double tol, int guess, int mixed, long long b0) {
  // b0: first block of a strip of cells (0 for the whole grid)
  k_newton_body<Sys, N>(VBlock{b0 + blockIdx.x, b0 + gridDim.x}, w, qh, g, T, wprod_g, st, tol, guess, mixed);
}

// ---------------------------------------------------------------------
// a9/a10/a12: face fluxes (fv.cpp:124-198, fluxes.cpp:72-117).  One
// thread per face point (direction d, face, time node t, transverse node
// idx).  Faces of direction d are indexed by their low-side w-cell O with
// O_d in [0, n_d] and O_e in [1, n_e] for e != d.  Writes
// tmp (b + f) and tmp (b - f), the amounts the reference subtracts from
// the low and high cell (fv.cpp:189-193).
// ---------------------------------------------------------------------
// The face state of transverse node idx: ENDVALS.row(e) * qh_ over the N
// nodes of its line along d (evaluations.cpp:49-70), rounded as the
// reference's Eigen GEMV rounds it (gemv_lane); the line's first node row
// lies off + base V doubles from the start of the reference's buffer.
template <class Sys, int N>
__device__ __forceinline__ void endpoints(const double *qhc, const Tables &T,
                                          int d, int e, int idx, double *out,
                                          long long off) {
  constexpr int V = Sys::V, D = Sys::NDIM;
  int sd = 1;
  for (int k = d + 1; k < D; k++)
    sd *= N;
  int hi = idx / sd, lo = idx % sd; // zero_index, evaluations.cpp:4-21
  int base = hi * sd * N + lo;
  const bool rot = gemv_rot(V, (long long)sd * V, off + (long long)base * V);
#pragma unroll
  for (int v = 0; v < V; v++)
    out[v] = gemv_lane(T.endvals + e * N, qhc + base * V + v, sd * V, N,
                       v < (V & ~1), rot);
}

template <class Sys, int N>
__device__ __forceinline__ void rusanov_flux(double *f, double *qL,
                                             double *qR, double *dqL,
                                             double *dqR, int d, double dXd) {
  constexpr int V = Sys::V;
  double fL[V], fR[V]; // F(qL), F(qR) come out of the FD Jacobians
  double m1, m2;
  if constexpr (V >= 6) { // a large system's eigen work spills when inlined twice
    m1 = max_abs_eigs_call<Sys>(qL, dqL, d, fL);
    m2 = max_abs_eigs_call<Sys>(qR, dqR, d, fR);
  } else {
    m1 = max_abs_eigs<Sys>(qL, dqL, d, fL);
    m2 = max_abs_eigs<Sys>(qR, dqR, d, fR);
  }
  double m = fmax(m1, m2);
#pragma unroll
  for (int v = 0; v < V; v++)
    f[v] = m * (qL[v] - qR[v]);
#pragma unroll
  for (int v = 0; v < V; v++)
    f[v] += fL[v] + fR[v];
  if (Sys::SECOND_ORDER) { // fluxes.cpp:96-100
    double a1 = max_abs_eigs_2nd<Sys>(qL, dqL, d, N, dXd);
    double a2 = max_abs_eigs_2nd<Sys>(qR, dqR, d, N, dXd);
    double mm = fmax(a1, a2);
#pragma unroll
    for (int v = 0; v < V; v++)
      f[v] += mm * (qL[v] - qR[v]);
  }
}

// |A| Dq from an eigen-decomposition A = R Lambda R^-1: solve R b = Dq,
// scale by |lambda|, multiply by R (fluxes.cpp:36-41, 64-69).  With
// accumulate, out += weight * that.
template <int V>
__device__ __noinline__ void abs_apply(const double *M, const double *Dq,
                                       double *out, double weight,
                                       bool accumulate) {
  double wr[V], wi[V], vr[V * V], vi[V * V];
  eig_full<V>(M, wr, wi, vr, vi);
  double mr[V * V], mi[V * V], br[V], bi[V];
  for (int i = 0; i < V * V; i++) {
    mr[i] = vr[i];
    mi[i] = vi[i];
  }
  for (int i = 0; i < V; i++) {
    br[i] = Dq[i];
    bi[i] = 0.0;
  }
  csolve<V>(mr, mi, br, bi);
  for (int i = 0; i < V; i++) {
    double l = sqrt(wr[i] * wr[i] + wi[i] * wi[i]);
    br[i] *= l;
    bi[i] *= l;
  }
  for (int i = 0; i < V; i++) {
    double s = 0;
    for (int j = 0; j < V; j++)
      s += vr[i * V + j] * br[j] - vi[i * V + j] * bi[j];
    out[i] = accumulate ? out[i] + weight * s : weight * s;
  }
}

// Osher: sum_i W_i |A(q_i)| (qL - qR) along the straight path
// q_i = qR + x_i (qL - qR) (fluxes.cpp:20-45).
template <class Sys, int N>
__device__ __forceinline__ void osher_d(double *ret, const double *qL,
                                        const double *qR, const double *dqL,
                                        const double *dqR, int d,
                                        const Tables &T) {
  constexpr int V = Sys::V, D = Sys::NDIM;
  double Dq[V], q[V], dq[D * V], M[V * V];
  for (int v = 0; v < V; v++) {
    Dq[v] = qL[v] - qR[v];
    ret[v] = 0.0;
  }
  for (int i = 0; i < N; i++) {
    for (int v = 0; v < V; v++)
      q[v] = qR[v] + T.nodes[i] * Dq[v];
    for (int k = 0; k < D * V; k++)
      dq[k] = dqR[k] + T.nodes[i] * (dqL[k] - dqR[k]);
    system_matrix<Sys>(M, q, dq, d);
    abs_apply<V>(M, Dq, ret, T.wghts[i], true);
  }
}

// Roe: |sum_i W_i A(q_i)| (qL - qR) (fluxes.cpp:47-70).
template <class Sys, int N>
__device__ __forceinline__ void roe_d(double *ret, const double *qL,
                                      const double *qR, const double *dqL,
                                      const double *dqR, int d,
                                      const Tables &T) {
  constexpr int V = Sys::V, D = Sys::NDIM;
  double Dq[V], q[V], dq[D * V], M[V * V], Mi[V * V];
  for (int v = 0; v < V; v++)
    Dq[v] = qL[v] - qR[v];
  for (int i = 0; i < V * V; i++)
    M[i] = 0.0;
  for (int i = 0; i < N; i++) {
    for (int v = 0; v < V; v++)
      q[v] = qR[v] + T.nodes[i] * Dq[v];
    for (int k = 0; k < D * V; k++)
      dq[k] = dqR[k] + T.nodes[i] * (dqL[k] - dqR[k]);
    system_matrix<Sys>(Mi, q, dq, d);
    for (int k = 0; k < V * V; k++)
      M[k] += T.wghts[i] * Mi[k];
  }
  abs_apply<V>(M, Dq, ret, 1.0, false);
}

// Roe / Osher numerical flux D + F(qL) + F(qR) (+ the second-order term),
// fluxes.cpp:80-101.
template <class Sys, int N, int FLUX>
__device__ __forceinline__ void eig_flux(double *f, double *qL, double *qR,
                                         double *dqL, double *dqR, int d,
                                         double dXd, const Tables &T) {
  constexpr int V = Sys::V;
  if (FLUX == 1)
    roe_d<Sys, N>(f, qL, qR, dqL, dqR, d, T);
  else
    osher_d<Sys, N>(f, qL, qR, dqL, dqR, d, T);
  double fL[V], fR[V];
  Sys::F(fL, qL, dqL, d);
  Sys::F(fR, qR, dqR, d);
#pragma unroll
  for (int v = 0; v < V; v++)
    f[v] += fL[v] + fR[v];
  if (Sys::SECOND_ORDER) {
    double a1 = max_abs_eigs_2nd<Sys>(qL, dqL, d, N, dXd);
    double a2 = max_abs_eigs_2nd<Sys>(qR, dqR, d, N, dXd);
    double mm = fmax(a1, a2);
#pragma unroll
    for (int v = 0; v < V; v++)
      f[v] += mm * (qL[v] - qR[v]);
  }
}

template <class Sys, int N>
__device__ __forceinline__ void bint(double *ret, const double *qL,
                                     const double *qR, int d,
                                     const Tables &T) {
  constexpr int V = Sys::V;
  double Dq[V], q[V], M[V * V], b[V * V];
#pragma unroll
  for (int v = 0; v < V; v++)
    Dq[v] = qR[v] - qL[v];
#pragma unroll
  for (int i = 0; i < V * V; i++)
    M[i] = 0.0;
  for (int i = 0; i < N; i++) {
#pragma unroll
    for (int v = 0; v < V; v++)
      q[v] = qL[v] + T.nodes[i] * Dq[v]; // fluxes.cpp:111-113
    Sys::B(b, q, d);
#pragma unroll
    for (int k = 0; k < V * V; k++)
      M[k] = M[k] + T.wghts[i] * b[k];
  }
#pragma unroll
  for (int r = 0; r < V; r++) {
    double s = 0;
#pragma unroll
    for (int j = 0; j < V; j++)
      s = fma(M[r * V + j], Dq[j], s);
    ret[r] = s;
  }
}

struct FaceIndex {
  long long off[4];   // first face point of each direction (off[D] = total)
  long long nface[3]; // faces per direction
};

// The face points one launch of k_faces covers: n[d] points of direction d
// from point lo[d] on.  A whole-grid launch has lo[d] = off[d] and
// n[d] = off[d+1] - off[d]; a strip launch has the points of the faces
// whose cells a set of predictor strips has finished.
struct FaceSpan {
  long long lo[3], n[3];
};

// Where face point p sits: its direction d, time node t, transverse node
// idx, and the qh offsets of its low- and high-side cells at time node t.
struct FaceAt {
  int d, t, idx;
  long long off0, off1;
};

template <class Sys, int N>
__device__ __forceinline__ FaceAt face_at(long long p, const Geom &g,
                                          const FaceIndex &fi) {
  constexpr int V = Sys::V, D = Sys::NDIM;
  constexpr int Nd = IPow<N, D>::value, Nd_ = IPow<N, D - 1>::value;
  FaceAt f;
  int d = 0;
  while (d + 1 < D && p >= fi.off[d + 1])
    d++;
  long long r = p - fi.off[d];
  f.d = d;
  f.idx = (int)(r % Nd_);
  r /= Nd_;
  f.t = (int)(r % N);
  long long face = r / N;
  // low-side w-cell O from the face index (row-major over the face box)
  int O[3];
  long long rem = face;
  for (int e = D - 1; e >= 0; e--) {
    int ext = (e == d) ? g.nX[e] + 1 : g.nX[e];
    int i = (int)(rem % ext);
    rem /= ext;
    O[e] = (e == d) ? i : i + 1;
  }
  long long qc0 = 0, qc1 = 0;
  for (int e = 0; e < D; e++) {
    qc0 = qc0 * g.nXw[e] + O[e];
    qc1 = qc1 * g.nXw[e] + O[e] + (e == d);
  }
  f.off0 = (qc0 * N + f.t) * (long long)Nd * V;
  f.off1 = (qc1 * N + f.t) * (long long)Nd * V;
  return f;
}

// The quadrature weight of a face point times dt / (2 dX_d) (fv.cpp:
// 176-193).
template <class Sys, int N>
__device__ __forceinline__ double face_weight(const FaceAt &f, double dt,
                                              const Geom &g, const Tables &T) {
  constexpr int D = Sys::NDIM;
  double tmp = dt * T.wghts[f.t] / (2. * g.dX[f.d]);
  int rm = f.idx;
  int dg[3] = {0, 0, 0};
  for (int e = D - 2; e >= 0; e--) {
    dg[e] = rm % N;
    rm /= N;
  }
  for (int e = 0; e < D - 1; e++)
    tmp *= T.wghts[dg[e]];
  return tmp;
}

// Face point p: its two face states, flux and path integral, and the
// amounts written to contrib[p].
template <class Sys, int N, int FLUX>
__device__ __forceinline__ void face_point(long long p, const double *__restrict__ qh, double *__restrict__ contrib,
            const Geom &g, const Tables &T, const FaceIndex &fi, double dt) {
  constexpr int V = Sys::V, D = Sys::NDIM;
  constexpr int Nd = IPow<N, D>::value;
  const FaceAt fa = face_at<Sys, N>(p, g, fi);
  const int d = fa.d, idx = fa.idx;
  const long long off0 = fa.off0, off1 = fa.off1;
  const double *qh0 = qh + off0;
  const double *qh1 = qh + off1;
  double q0[V], q1[V], dq0[D * V], dq1[D * V];
  endpoints<Sys, N>(qh0, T, d, 1, idx, q0, off0);
  endpoints<Sys, N>(qh1, T, d, 0, idx, q1, off1);
#pragma unroll
  for (int k = 0; k < D * V; k++)
    dq0[k] = dq1[k] = 0.0;
  if (Sys::SECOND_ORDER) {
    // gradients at the face point: endpoints of derivs of qh
    // (fv.cpp:87-122), both rounded as the reference rounds them; its
    // dqh stacks one qh-shaped block per direction d_
    double tmpd[Nd * V];
    for (int d_ = 0; d_ < D; d_++) {
      for (int side = 0; side < 2; side++) {
        const double *src = side ? qh1 : qh0;
        int sd = 1;
        for (int e = d_ + 1; e < D; e++)
          sd *= N;
        for (int n = 0; n < Nd; n++) {
          int id = (n / sd) % N;
          int base = n - id * sd;
          for (int v = 0; v < V; v++) {
            double s = 0;
            for (int j = 0; j < N; j++)
              s = s + T.dervals[id * N + j] * src[(base + j * sd) * V + v];
            tmpd[n * V + v] = s / g.dX[d_];
          }
        }
        double e_out[V];
        const long long offd = d_ * g.Cw * (long long)(N * Nd * V);
        endpoints<Sys, N>(tmpd, T, d, side ? 0 : 1, idx, e_out,
                          offd + (side ? off1 : off0));
        for (int v = 0; v < V; v++)
          (side ? dq1 : dq0)[d_ * V + v] = e_out[v];
      }
    }
  }
  double f[V], b[V];
#pragma unroll
  for (int v = 0; v < V; v++)
    f[v] = b[v] = 0.0;
  if (Sys::HAS_F) {
    if (FLUX == 0)
      rusanov_flux<Sys, N>(f, q0, q1, dq0, dq1, d, g.dX[d]);
    else
      eig_flux<Sys, N, FLUX>(f, q0, q1, dq0, dq1, d, g.dX[d], T);
  }
  if (Sys::HAS_B)
    bint<Sys, N>(b, q0, q1, d, T);
  const double tmp = face_weight<Sys, N>(fa, dt, g, T);
  double *o = contrib + p * 2 * V;
#pragma unroll
  for (int v = 0; v < V; v++) {
    o[v] = tmp * (b[v] + f[v]);
    o[V + v] = tmp * (b[v] - f[v]);
  }
}

// Face point q of a launch's span (direction by direction).
__device__ __forceinline__ long long span_point(const FaceSpan &sp, int D,
                                                long long q) {
  int d = 0;
  while (d + 1 < D && q >= sp.n[d])
    q -= sp.n[d++];
  return sp.lo[d] + q;
}

// ---------------------------------------------------------------------
// The Rusanov faces of a first-order flux system without B in two
// launches.  Alone, the face kernel needs 255 registers a thread: the face
// states and fluxes stay live across the eigenvalue solves, which need
// about 127 of their own.  Split, k_faces_pre (states, F, the FD
// Jacobians) and k_faces_eig (max|eig|, the Rusanov flux, contrib) each
// need far fewer, and an SM holds twice the warps.  k_faces_pre writes, per
// face point j of a chunk, a record of REC doubles, component-major with
// stride ch (coalesced):
//   [0, MS^2)        the matrix max_abs_eig takes at the low-side state
//   [MS^2, 2 MS^2)   the same at the high-side state
//   qL (V), qR (V), fL + fR (V), the face weight, ok (1 + 2: the low /
//   high side's matrix is the active block of max_abs_eigs, else
//   k_faces_eig runs max_abs_eigs on the state itself)
// Every value is computed by the same operations as in face_point, so the
// results are the same bits.
// ---------------------------------------------------------------------
template <class S, class = void> struct EigBlock {
  static constexpr int value = S::V;
};
template <class S>
struct EigBlock<S, void_t_<decltype(S::EIG_ACTIVE)>> {
  static constexpr int value = S::EIG_ACTIVE;
};

template <class Sys> struct FaceSplit {
  static constexpr bool OK = Sys::HAS_F && !Sys::HAS_B && !Sys::SECOND_ORDER;
  static constexpr int MS = EigBlock<Sys>::value;
  static constexpr int REC = 2 * MS * MS + 3 * Sys::V + 2;
  // CTAs an SM that k_faces_eig is compiled for: 6 (80 registers) for a
  // 5x5 block, where max_abs_eig<5> then spills and the stage is still
  // faster (2-D relaxation system at 1024^2: 31.7 ms a step against 32.1
  // with 4 CTAs and 32.2 with 5); 4 (128 registers, no spills in the
  // solver) otherwise
  static constexpr int EIG_CTAS = MS == 5 ? 6 : 4;
};

// The first half of max_abs_eigs: the matrix max_abs_eig takes and F(q)
// in f0.  False when a system's active block does not apply (its passive
// rows are not zero); max_abs_eigs must then run on q itself.
template <class Sys>
__device__ __forceinline__ bool eig_matrix(double *S, double *q, double *dq,
                                           int d, double *f0) {
  if constexpr (HasEigActive<Sys>::value) {
    return fd_jacobian_active<Sys>(S, q, dq, d, f0);
  } else {
    fd_jacobian<Sys>(S, q, dq, d, false, f0);
    return true;
  }
}

// The record of face point p at r, components ch apart.
template <class Sys, int N>
__device__ __forceinline__ void face_pre_point(long long p, const double *__restrict__ qh,
                                               double *r, long long ch, const Geom &g,
                                               const Tables &T, const FaceIndex &fi,
                                               double dt) {
  constexpr int V = Sys::V, D = Sys::NDIM, MS = FaceSplit<Sys>::MS;
  const FaceAt fa = face_at<Sys, N>(p, g, fi);
  double q[V], dq[D * V], S[MS * MS], fL[V], fR[V];
#pragma unroll
  for (int k = 0; k < D * V; k++)
    dq[k] = 0.0;
  // one side at a time, each written out before the next is formed
  endpoints<Sys, N>(qh + fa.off0, T, fa.d, 1, fa.idx, q, fa.off0);
  const bool okL = eig_matrix<Sys>(S, q, dq, fa.d, fL);
#pragma unroll
  for (int k = 0; k < MS * MS; k++)
    r[k * ch] = S[k];
  double *rs = r + 2 * MS * MS * ch;
#pragma unroll
  for (int v = 0; v < V; v++)
    rs[v * ch] = q[v];
  endpoints<Sys, N>(qh + fa.off1, T, fa.d, 0, fa.idx, q, fa.off1);
  const bool okR = eig_matrix<Sys>(S, q, dq, fa.d, fR);
#pragma unroll
  for (int k = 0; k < MS * MS; k++)
    r[(MS * MS + k) * ch] = S[k];
#pragma unroll
  for (int v = 0; v < V; v++) {
    rs[(V + v) * ch] = q[v];
    rs[(2 * V + v) * ch] = fL[v] + fR[v];
  }
  rs[3 * V * ch] = face_weight<Sys, N>(fa, dt, g, T);
  rs[(3 * V + 1) * ch] = (double)((okL ? 1 : 0) + (okR ? 2 : 0));
}

// Points [q0, q0 + min(ch, total - q0)) of span sp.
template <class Sys, int N>
__global__ void __launch_bounds__(128)
    k_faces_pre(const double *__restrict__ qh, double *__restrict__ rec, long long ch,
                const __grid_constant__ Geom g, const __grid_constant__ Tables T,
                const __grid_constant__ FaceIndex fi, DevState *st,
                const __grid_constant__ FaceSpan sp, long long q0) {
  if (!step_active(st))
    return;
  const double dt = st->dt;
  const long long total = sp.n[0] + sp.n[1] + sp.n[2];
  const long long n = (total - q0 < ch) ? total - q0 : ch;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x)
    face_pre_point<Sys, N>(span_point(sp, Sys::NDIM, q0 + j), qh, rec + j, ch, g,
                           T, fi, dt);
}

// max_abs_eigs on a face state read from a record (the rare side whose
// active block did not apply), out of line so that the eigenvalue kernel
// keeps no state for it.
template <class Sys>
__device__ __noinline__ double max_abs_eigs_rec(const double *rq, long long ch,
                                                int d) {
  constexpr int V = Sys::V, D = Sys::NDIM;
  double q[V], dq[D * V];
  for (int v = 0; v < V; v++)
    q[v] = rq[v * ch];
  for (int k = 0; k < D * V; k++)
    dq[k] = 0.0;
  return max_abs_eigs<Sys>(q, dq, d);
}

// Face point p from its record at r (components ch apart): max|eig| on
// both sides, the Rusanov flux (fluxes.cpp:86-101, as rusanov_flux) and
// contrib[p].
template <class Sys, int N>
__device__ __forceinline__ void face_eig_point(long long p, const double *r, long long ch,
                                               double *__restrict__ contrib,
                                               const FaceIndex &fi) {
  constexpr int V = Sys::V, D = Sys::NDIM, MS = FaceSplit<Sys>::MS;
  int d = 0;
  while (d + 1 < D && p >= fi.off[d + 1])
    d++;
  const double *rs = r + 2 * MS * MS * ch;
  const int ok = (int)rs[(3 * V + 1) * ch];
  double m1, m2;
  {
    double S[MS * MS];
#pragma unroll
    for (int k = 0; k < MS * MS; k++)
      S[k] = r[k * ch];
    m1 = (ok & 1) ? max_abs_eig<MS>(S) : max_abs_eigs_rec<Sys>(rs, ch, d);
  }
  {
    double S[MS * MS];
#pragma unroll
    for (int k = 0; k < MS * MS; k++)
      S[k] = r[(MS * MS + k) * ch];
    m2 = (ok & 2) ? max_abs_eig<MS>(S)
                  : max_abs_eigs_rec<Sys>(rs + V * ch, ch, d);
  }
  const double m = fmax(m1, m2);
  const double tmp = rs[3 * V * ch];
  double f[V], b[V];
#pragma unroll
  for (int v = 0; v < V; v++) {
    b[v] = 0.0;
    f[v] = m * (rs[v * ch] - rs[(V + v) * ch]);
  }
#pragma unroll
  for (int v = 0; v < V; v++)
    f[v] += rs[(2 * V + v) * ch];
  double *o = contrib + p * 2 * V;
#pragma unroll
  for (int v = 0; v < V; v++) {
    o[v] = tmp * (b[v] + f[v]);
    o[V + v] = tmp * (b[v] - f[v]);
  }
}

// The records of k_faces_pre for the same points, FaceSplit<Sys>::EIG_CTAS
// CTAs an SM.
template <class Sys, int N>
__global__ void __launch_bounds__(128, FaceSplit<Sys>::EIG_CTAS)
    k_faces_eig(const double *__restrict__ rec, long long ch, double *__restrict__ contrib,
                const __grid_constant__ FaceIndex fi, DevState *st,
                const __grid_constant__ FaceSpan sp, long long q0) {
  if (!step_active(st))
    return;
  const long long total = sp.n[0] + sp.n[1] + sp.n[2];
  const long long n = (total - q0 < ch) ? total - q0 : ch;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x)
    face_eig_point<Sys, N>(span_point(sp, Sys::NDIM, q0 + j), rec + j, ch, contrib,
                           fi);
}

// Every face point of the grid (one tile of a batched launch).
template <class Sys, int N, int FLUX>
__device__ __forceinline__ void k_faces_body(VBlock vb_, const double *__restrict__ qh, double *__restrict__ contrib,
            const Geom &g, const Tables &T, const FaceIndex &fi, DevState *st) {
  if (!step_active(st))
    return;
  const double dt = st->dt;
  for (long long p = vb_.b * (long long)blockDim.x + threadIdx.x;
       p < fi.off[Sys::NDIM]; p += (long long)vb_.n * blockDim.x)
    face_point<Sys, N, FLUX>(p, qh, contrib, g, T, fi, dt);
}

// The face points of span sp, direction by direction.
template <class Sys, int N, int FLUX = 0>
__global__ void __launch_bounds__(128)
    k_faces(const double *__restrict__ qh, double *__restrict__ contrib,
            const __grid_constant__ Geom g, const __grid_constant__ Tables T, const __grid_constant__ FaceIndex fi, DevState *st,
            const __grid_constant__ FaceSpan sp) {
  if (!step_active(st))
    return;
  const double dt = st->dt;
  long long total = 0;
  for (int d = 0; d < Sys::NDIM; d++)
    total += sp.n[d];
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x)
    face_point<Sys, N, FLUX>(span_point(sp, Sys::NDIM, q), qh, contrib, g, T, fi, dt);
}

// ---------------------------------------------------------------------
// a8: centre (volume) terms, fv.cpp:33-85.  One thread per (u-cell,
// space-time node): dt W_t prod W (S(qh) - sum_d B_d dqh_d).
// ---------------------------------------------------------------------
template <class Sys, int N>
__device__ __forceinline__ void k_centers_body(VBlock vb_, const double *__restrict__ qh,
                          double *__restrict__ cen, const Geom &g, const Tables &T,
                          DevState *st) {
  constexpr int V = Sys::V, D = Sys::NDIM;
  constexpr int Nd = IPow<N, D>::value, NT = N * Nd;
  if (!step_active(st))
    return;
  const double dt = st->dt;
  long long total = g.C * NT;
  for (long long e = vb_.b * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)vb_.n * blockDim.x) {
    long long uc = e / NT;
    int node = (int)(e % NT);
    int t = node / Nd, idx = node % Nd;
    long long rem = uc, rc = 0, mul = 1;
    for (int d = D - 1; d >= 0; d--) {
      int i = (int)(rem % g.nX[d]);
      rem /= g.nX[d];
      rc += mul * (i + 1);
      mul *= g.nXw[d];
    }
    const double *qt = qh + (rc * N + t) * (long long)Nd * V;
    int digs[3] = {0, 0, 0};
    {
      int rm = idx;
      for (int d = D - 1; d >= 0; d--) {
        digs[d] = rm % N;
        rm /= N;
      }
    }
    double s[V];
    if (Sys::HAS_S)
      Sys::S(s, qt + idx * V);
    else
#pragma unroll
      for (int v = 0; v < V; v++)
        s[v] = 0.0;
    if (Sys::HAS_B) {
#pragma unroll
      for (int d = 0; d < D; d++) {
        int sd = 1;
        for (int k = d + 1; k < D; k++)
          sd *= N;
        int base = idx - digs[d] * sd;
        double dq[V], b[V * V];
#pragma unroll
        for (int v = 0; v < V; v++) {
          double a = 0;
#pragma unroll
          for (int j = 0; j < N; j++)
            a = fma(T.dervals[digs[d] * N + j], qt[(base + j * sd) * V + v], a);
          dq[v] = a * (1.0 / g.dX[d]);
        }
        Sys::B(b, qt + idx * V, d);
#pragma unroll
        for (int i = 0; i < V; i++) {
          double acc = 0;
#pragma unroll
          for (int j = 0; j < V; j++)
            acc = fma(b[i * V + j], dq[j], acc);
          s[i] -= acc;
        }
      }
    }
    double tmp = dt * T.wghts[t];
    for (int d = 0; d < D; d++)
      tmp *= T.wghts[digs[d]];
    double *o = cen + e * V;
#pragma unroll
    for (int v = 0; v < V; v++)
      o[v] = tmp * s[v];
  }
}

template <class Sys, int N>
__global__ void k_centers(const double *__restrict__ qh,
                          double *__restrict__ cen, const __grid_constant__ Geom g, const __grid_constant__ Tables T,
                          DevState *st) {
  k_centers_body<Sys, N>(VBlock{(long long)blockIdx.x, (long long)gridDim.x}, qh, cen, g, T, st);
}

// ---------------------------------------------------------------------
// Apply centre and face contributions to u in the order the reference's
// loops do (fv.cpp:200-207: centres first, then the face loop over the
// low-side w-cell O in row-major order with t, then d, then idx inside):
// for u-cell c at w-index C, the faces with O = C - e_0, ..., C - e_{D-1}
// (c is their high side) come before O = C (c is the low side of all D).
// One thread per (u-cell, variable).  Also flags NaN (iterator.cpp:141).
// ---------------------------------------------------------------------
template <class Sys, int N>
__device__ __forceinline__ void k_gather_body(VBlock vb_, double *__restrict__ u, const double *__restrict__ cen,
                         const double *__restrict__ contrib, const Geom &g,
                         const FaceIndex &fi, int use_centers, int use_faces,
                         DevState *st) {
  constexpr int V = Sys::V, D = Sys::NDIM;
  constexpr int Nd = IPow<N, D>::value, Nd_ = IPow<N, D - 1>::value;
  if (!step_active(st))
    return;
  long long total = g.C * V;
  bool nan_seen = false;
  for (long long e = vb_.b * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)vb_.n * blockDim.x) {
    long long uc = e / V;
    int v = (int)(e % V);
    double val = u[e];
    if (use_centers) {
      const double *c = cen + uc * (N * Nd) * V + v;
      for (int k = 0; k < N * Nd; k++)
        val += c[k * V];
    }
    if (use_faces) {
      int ic[3];
      long long rem = uc;
      for (int d = D - 1; d >= 0; d--) {
        ic[d] = (int)(rem % g.nX[d]);
        rem /= g.nX[d];
      }
      // as the high side of the face with O = C - e_dd, for dd = 0..D-1
      for (int dd = 0; dd < D; dd++) {
        long long face = 0;
        for (int e2 = 0; e2 < D; e2++) {
          int ext = (e2 == dd) ? g.nX[e2] + 1 : g.nX[e2];
          int oi = (e2 == dd) ? ic[e2] : ic[e2]; // O_e - (e != dd ? 1 : 0)
          face = face * ext + oi;
        }
        const double *c = contrib + (fi.off[dd] + face * N * Nd_) * 2 * V;
        for (int t = 0; t < N; t++)
          for (int idx = 0; idx < Nd_; idx++)
            val -= c[((t * Nd_ + idx) * 2 + 1) * V + v];
      }
      // as the low side (O = C) of all D faces, t outer, d inner
      long long facel[3];
      for (int dd = 0; dd < D; dd++) {
        long long face = 0;
        for (int e2 = 0; e2 < D; e2++) {
          int ext = (e2 == dd) ? g.nX[e2] + 1 : g.nX[e2];
          int oi = (e2 == dd) ? ic[e2] + 1 : ic[e2];
          face = face * ext + oi;
        }
        facel[dd] = face;
      }
      for (int t = 0; t < N; t++)
        for (int dd = 0; dd < D; dd++) {
          const double *c =
              contrib + (fi.off[dd] + (facel[dd] * N + t) * Nd_) * 2 * V;
          for (int idx = 0; idx < Nd_; idx++)
            val -= c[(idx * 2) * V + v];
        }
    }
    u[e] = val;
    if (!(val == val))
      nan_seen = true;
  }
  if (__syncthreads_or(nan_seen) && threadIdx.x == 0)
    atomicOr(&st->nan_now, 1);
}

template <class Sys, int N>
__global__ void k_gather(double *__restrict__ u, const double *__restrict__ cen,
                         const double *__restrict__ contrib, const __grid_constant__ Geom g,
                         const __grid_constant__ FaceIndex fi, int use_centers, int use_faces,
                         DevState *st) {
  k_gather_body<Sys, N>(VBlock{(long long)blockIdx.x, (long long)gridDim.x}, u, cen, contrib, g, fi, use_centers, use_faces, st);
}

} // namespace pypde
