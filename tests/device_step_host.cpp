// The whole ADER-WENO step of pypde_gb300/csrc (ghost fill, WENO passes,
// CFL reduction, Picard and Newton predictors, face fluxes, centres and the
// gather) compiled as host C++ and run with every CUDA thread of a block
// emulated by a fiber, for a CPU test that compares it bit for bit with
// the C restatement.
//
// The emulation:
// - blocks of a launch run one after the other; the CUDA threads of a block
//   are ucontext fibers on one host thread, each run until it reaches a
//   barrier or returns; `__shared__` is `static` here, so shared memory is
//   shared by the fibers of the block;
// - __syncthreads, __syncthreads_and and __syncthreads_or release the block
//   once every thread that has not returned waits there, with the AND/OR
//   of the predicate; a thread that returned takes no part, as an exited
//   thread on the GPU;
// - __syncwarp(mask) releases the lanes of `mask` once every one of them
//   that has not returned waits at a warp barrier with that mask (the full
//   mask: the whole warp), and __shfl_down_sync exchanges values through a
//   per-warp buffer between two full-warp barriers;
// - a block whose threads wait at barriers that can never all be released
//   (some lanes of a warp at a warp barrier, others at the block barrier)
//   is reported as a deadlock;
// - the fibers run in thread order or in reverse order (host_set_order):
//   a result that changes with the order shows a read of shared memory
//   that no barrier orders after its write;
// - the kernels' dynamic shared memory is a buffer sized by the same
//   configuration constant the runtime passes at launch.
// The test copies the headers of pypde_gb300/csrc into a build folder and
// replaces each `extern __shared__ double smem[];` by a call of
// host_dynamic_smem() below (a host compiler cannot declare a static
// array of unknown size); nothing else in them is changed.
//
// The launch shapes (grid and block sizes) and the stage order follow the
// one-problem step of pypde_gb300/csrc/runtime.cu (enqueue_step,
// enqueue_weno, enqueue_predictor) and its batched step (run_batch,
// enqueue_batch_step: the kb_* kernels of batch.cuh over a tile queue).
#include <ucontext.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

// Entry points are the only exported symbols: the unit is built with hidden
// visibility and without GNU unique symbols, so that the block-shared
// statics of two of these libraries loaded into one process (two run-time
// systems, each a `UserSystem`) stay apart.
#define HOST_API extern "C" __attribute__((visibility("default")))

#define __device__
#define __host__
#define __global__
#define __shared__ static
#define __grid_constant__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __launch_bounds__(...)

struct HostDim3 {
  unsigned x, y, z;
};
static HostDim3 threadIdx, blockIdx, blockDim, gridDim;

namespace emu {

enum State { RUNNABLE, AT_BLOCK, AT_WARP, DONE };

struct Fiber {
  ucontext_t ctx;
  char *stack = nullptr;
  State state = DONE;
  int pred = 0;
  unsigned wmask = 0xffffffffu; // lanes of the warp barrier it waits at
  unsigned long long slot = 0;   // shuffle buffer
};

constexpr size_t STACK_BYTES = 512 * 1024;
static ucontext_t g_sched;
static std::vector<Fiber> g_f;
static const std::function<void()> *g_body = nullptr;
static unsigned g_cur = 0, g_n = 0;
static int g_red_and = 1, g_red_or = 0;
static bool g_reverse = false;
static bool g_deadlock = false;
static std::vector<double> g_smem;

static void trampoline(int i) {
  (*g_body)();
  g_f[i].state = DONE;
} // returns to uc_link, the scheduler

// Suspends the current fiber in state s until the scheduler releases it.
static void wait_in(State s) {
  g_f[g_cur].state = s;
  swapcontext(&g_f[g_cur].ctx, &g_sched);
  threadIdx = HostDim3{g_cur, 0, 0};
}

static int block_sync(int p, int mode) {
  g_f[g_cur].pred = p != 0;
  wait_in(AT_BLOCK);
  return mode == 1 ? g_red_and : (mode == 2 ? g_red_or : 0);
}

static void run_block(unsigned n) {
  if (g_f.size() < n)
    g_f.resize(n);
  for (unsigned i = 0; i < n; i++) {
    Fiber &f = g_f[i];
    if (!f.stack)
      f.stack = static_cast<char *>(std::malloc(STACK_BYTES));
    getcontext(&f.ctx);
    f.ctx.uc_stack.ss_sp = f.stack;
    f.ctx.uc_stack.ss_size = STACK_BYTES;
    f.ctx.uc_link = &g_sched;
    makecontext(&f.ctx, (void (*)())trampoline, 1, (int)i);
    f.state = RUNNABLE;
  }
  g_n = n;
  for (;;) {
    for (unsigned k = 0; k < n; k++) {
      const unsigned i = g_reverse ? n - 1 - k : k;
      if (g_f[i].state != RUNNABLE)
        continue;
      g_cur = i;
      threadIdx = HostDim3{i, 0, 0};
      swapcontext(&g_sched, &g_f[i].ctx);
    }
    // every fiber now waits at a barrier or has returned
    bool released = false;
    for (unsigned w0 = 0; w0 < n; w0 += 32) {
      const unsigned w1 = w0 + 32 < n ? w0 + 32 : n;
      for (unsigned i = w0; i < w1; i++) {
        if (g_f[i].state != AT_WARP)
          continue;
        // every lane of i's mask that has not returned waits with it
        const unsigned m = g_f[i].wmask;
        bool all = true;
        for (unsigned j = w0; j < w1; j++) {
          if (!(m >> (j - w0) & 1u) || g_f[j].state == DONE)
            continue;
          if (g_f[j].state != AT_WARP || g_f[j].wmask != m)
            all = false;
        }
        if (!all)
          continue;
        for (unsigned j = w0; j < w1; j++)
          if ((m >> (j - w0) & 1u) && g_f[j].state == AT_WARP)
            g_f[j].state = RUNNABLE;
        released = true;
      }
    }
    if (released)
      continue;
    int live = 0, at = 0, a = 1, o = 0;
    for (unsigned i = 0; i < n; i++)
      if (g_f[i].state != DONE) {
        live++;
        if (g_f[i].state == AT_BLOCK) {
          at++;
          a &= g_f[i].pred;
          o |= g_f[i].pred;
        }
      }
    if (live == 0)
      return;
    if (at != live) {
      g_deadlock = true; // the waiting fibers are abandoned
      return;
    }
    g_red_and = a;
    g_red_or = o;
    for (unsigned i = 0; i < n; i++)
      if (g_f[i].state == AT_BLOCK)
        g_f[i].state = RUNNABLE;
  }
}

// Runs body once per CUDA thread of a grid x block launch; blocks run in
// order.
static void launch(unsigned grid, unsigned block, size_t smem_bytes,
                   const std::function<void()> &body) {
  gridDim = HostDim3{grid, 1, 1};
  blockDim = HostDim3{block, 1, 1};
  g_smem.assign(smem_bytes / 8 + 1, 0.0);
  g_body = &body;
  for (unsigned b = 0; b < grid && !g_deadlock; b++) {
    blockIdx = HostDim3{b, 0, 0};
    run_block(block);
  }
}

} // namespace emu

static double *host_dynamic_smem() { return emu::g_smem.data(); }

static inline void __syncthreads() { emu::block_sync(1, 0); }
static inline int __syncthreads_and(int p) { return emu::block_sync(p, 1); }
static inline int __syncthreads_or(int p) { return emu::block_sync(p, 2); }
static inline void __syncwarp(unsigned mask = 0xffffffffu) {
  emu::g_f[threadIdx.x].wmask = mask;
  emu::wait_in(emu::AT_WARP);
}
template <class T> static inline T __shfl_down_sync(unsigned, T v, int off) {
  static_assert(sizeof(T) <= 8, "shuffle of a wider type");
  const unsigned lane = threadIdx.x % 32, base = threadIdx.x - lane;
  std::memcpy(&emu::g_f[threadIdx.x].slot, &v, sizeof(T));
  emu::g_f[threadIdx.x].wmask = 0xffffffffu;
  emu::wait_in(emu::AT_WARP);
  T r = v;
  const unsigned src = base + lane + off;
  if (lane + off < 32 && src < emu::g_n)
    std::memcpy(&r, &emu::g_f[src].slot, sizeof(T));
  emu::wait_in(emu::AT_WARP);
  return r;
}
// One host thread runs every fiber and a fiber is never suspended inside
// an atomic, so a plain read-modify-write is atomic here.
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
static inline unsigned __float_as_uint(float x) {
  unsigned r;
  std::memcpy(&r, &x, sizeof r);
  return r;
}
static inline float __uint_as_float(unsigned x) {
  float r;
  std::memcpy(&r, &x, sizeof r);
  return r;
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
template <class T> static inline T max(T a, T b) { return a > b ? a : b; }
template <class T> static inline T min(T a, T b) { return a < b ? a : b; }

using std::exp;
using std::fabs;
using std::fma;
using std::fmax;
using std::fmin;
using std::log;
using std::pow;
using std::sqrt;

#include "step_kernels.cuh"
#include "strips.h"
#include "systems.cuh"

namespace {
using namespace pypde;

unsigned grid_for(long long work, int threads, int cap_blocks) {
  long long b = (work + threads - 1) / threads;
  if (b < 1)
    b = 1;
  if (b > cap_blocks)
    b = cap_blocks;
  return (unsigned)b;
}

int ipow(int b, int e) {
  int r = 1;
  while (e-- > 0)
    r *= b;
  return r;
}

// The tables in the packed order of pypde_tables (nodes, weights, DERVALS,
// ENDVALS, DG_MAT, its inverse, the four WENO inverses, Sigma).
Tables unpack_tables(int N, const double *p) {
  Tables T;
  std::memset(&T, 0, sizeof T);
  T.N = N;
  auto get = [&](double *dst, int n) {
    std::memcpy(dst, p, sizeof(double) * n);
    p += n;
  };
  get(T.nodes, N);
  get(T.wghts, N);
  get(T.dervals, N * N);
  get(T.endvals, 2 * N);
  get(T.dgmat, N * N);
  get(T.dgmat_inv, N * N);
  for (int k = 0; k < 4; k++)
    get(T.weno_inv[k], N * N);
  get(T.sig, N * N);
  return T;
}

// Host set-up of one problem, as pypde_gb300/csrc/runtime.cu does it.
Geom make_geom(int ndim, const int *nX, const int *bt, const double *dX,
               int N) {
  Geom g;
  std::memset(&g, 0, sizeof(g));
  g.ndim = ndim;
  g.C = g.Cb = g.Cw = 1;
  for (int d = 0; d < 3; d++) {
    bool in = d < ndim;
    g.nX[d] = in ? nX[d] : 1;
    g.nXb[d] = in ? nX[d] + 2 * N : 1;
    g.nXw[d] = in ? nX[d] + 2 : 1;
    g.bt[d] = in && bt ? bt[d] : 0;
    g.dX[d] = in && dX ? dX[d] : 1.0;
    if (in) {
      g.C *= g.nX[d];
      g.Cb *= g.nXb[d];
      g.Cw *= g.nXw[d];
    }
  }
  return g;
}

FaceIndex make_face_index(const Geom &g, int N) {
  FaceIndex fi;
  std::memset(&fi, 0, sizeof(fi));
  long long Nd_ = 1;
  for (int d = 0; d < g.ndim - 1; d++)
    Nd_ *= N;
  for (int d = 0; d < 3; d++) {
    if (d < g.ndim) {
      long long nf = g.nX[d] + 1;
      for (int e = 0; e < g.ndim; e++)
        if (e != d)
          nf *= g.nX[e];
      fi.nface[d] = nf;
      fi.off[d + 1] = fi.off[d] + nf * N * Nd_;
    } else {
      fi.off[d + 1] = fi.off[d];
    }
  }
  return fi;
}

std::vector<double> make_wprod(const Tables &T, int ndim) {
  const int N = T.N, Nd = ipow(N, ndim);
  std::vector<double> wp(Nd);
  for (int idx = 0; idx < Nd; idx++) {
    int digs[3] = {0, 0, 0}, r = idx;
    for (int d = ndim - 1; d >= 0; d--) {
      digs[d] = r % N;
      r /= N;
    }
    double p = 1.0;
    for (int d = 0; d < ndim; d++)
      p *= T.wghts[digs[d]];
    wp[idx] = p;
  }
  return wp;
}

// The predictor stage of one step: Picard (k_predictor) or Newton
// (k_newton), launched as enqueue_predictor does.
// With guess = 1 the Newton iteration starts from the qh already given.
// Blocks [b_lo, b_hi) only (a strip of cells) when b_hi >= 0.
template <class Sys, int N>
void predictor_stage(bool stiff, const double *w, double *qh, const Geom &g,
                     const Tables &T, const double *wprod, DevState *st,
                     double tol, int mixed, int guess = 0, long long b_lo = 0,
                     long long b_hi = -1) {
  if (stiff) {
    using NC = NewtonCfg<Sys, N>;
    if (b_hi < 0)
      b_hi = (g.Cw + NC::CPB - 1) / NC::CPB;
    if (b_hi <= b_lo)
      return;
    emu::launch((unsigned)(b_hi - b_lo), NC::THREADS, NC::SMEM_BYTES, [&] {
      k_newton<Sys, N>(w, qh, g, T, wprod, st, tol, guess, mixed, b_lo);
    });
  } else {
    using PC = PredCfg<Sys, N>;
    if (b_hi < 0)
      b_hi = (g.Cw + PC::CPB - 1) / PC::CPB;
    if (b_hi <= b_lo)
      return;
    emu::launch((unsigned)(b_hi - b_lo), PC::THREADS,
                (size_t)PC::SMEM_DOUBLES * 8,
                [&] { k_predictor<Sys, N>(w, qh, g, T, wprod, st, b_lo); });
  }
}

// Strips of the step (as run_solver plans them; 1: one launch each).  The
// emulation runs strip i's faces right after strip i's predictor, before
// strip i+1 is predicted, so a face that read a cell of a later strip
// would read last step's qh (or zeros) and miss the restatement.
int g_strips = 1;

// Steps of the one-problem run, in the order of enqueue_step, until the
// step is inactive (t >= tf, the step cap, or a NaN).  Returns the steps
// taken.
template <class Sys, int N, int FLUX>
long long run_steps(double *u, int ndim, const int *nX, const int *bt,
                    const double *dX, const double *tabs, double tf,
                    double cfl, int stiff, double tol, int mixed,
                    long long max_steps, double *t_out,
                    unsigned long long *iters_out) {
  constexpr int V = Sys::V;
  const Tables T = unpack_tables(N, tabs);
  const Geom g = make_geom(ndim, nX, bt, dX, N);
  const FaceIndex fi = make_face_index(g, N);
  const int Nd = ipow(N, ndim);
  const bool faces = Sys::HAS_F || Sys::HAS_B;
  const bool centers = Sys::HAS_B || Sys::HAS_S;
  std::vector<double> uprev(g.C * V), ub(g.Cb * V), w(g.Cw * Nd * V),
      qh(g.Cw * N * Nd * V), contrib((faces ? fi.off[ndim] : 1) * 2 * V),
      cen((centers ? g.C * N * Nd : 1) * V);
  long long tmpn = 1;
  {
    int m[3];
    for (int d = 0; d < ndim; d++)
      m[d] = g.nXb[d];
    long long n4 = 1;
    for (int d = 0; d < ndim - 1; d++) {
      m[d] -= 2 * (N - 1);
      n4 *= N;
      long long sz = n4 * V;
      for (int e = 0; e < ndim; e++)
        sz *= m[e];
      if (sz > tmpn)
        tmpn = sz;
    }
  }
  std::vector<double> tmpA(tmpn), tmpB(tmpn);
  const std::vector<double> wprod = make_wprod(T, ndim);
  DevState st;
  std::memset(&st, 0, sizeof(st));
  st.tf = tf;
  st.cfl = cfl;
  st.max_steps = max_steps > 0 ? max_steps : -1;
  st.ndt = 1;
  st.snap_slot = -1;
  for (;;) {
    step_begin_dev(&st);
    if (!st.active || emu::g_deadlock)
      break;
    const long long n = g.C * V;
    emu::launch(grid_for(n, 256, 152 * 16), 256, 0,
                [&] { k_copy_prev(u, uprev.data(), n, &st); });
    emu::launch(grid_for(g.Cb * V, 256, 152 * 32), 256, 0,
                [&] { k_boundaries(u, ub.data(), g, N, V, &st); });
    {
      int m[3];
      for (int d = 0; d < ndim; d++)
        m[d] = g.nXb[d];
      const double *src = ub.data();
      int n4 = 1;
      for (int d = 0; d < ndim; d++) {
        long long n1 = 1, n3 = 1;
        for (int e = 0; e < d; e++)
          n1 *= m[e];
        for (int e = d + 1; e < ndim; e++)
          n3 *= m[e];
        const int md = m[d];
        double *dst = (d == ndim - 1) ? w.data()
                                      : ((d % 2 == 0) ? tmpA.data() : tmpB.data());
        const long long total = n1 * (md - 2 * (N - 1)) * n3 * (long long)n4 * V;
        emu::launch(grid_for(total, 128, 152 * 64), 128, 0, [&] {
          k_weno_pass<N>(src, dst, n1, md, n3, n4, V, T, &st);
        });
        src = dst;
        m[d] -= 2 * (N - 1);
        n4 *= N;
      }
    }
    emu::launch(grid_for(g.Cw, 128, 152 * 64), 128, 0, [&] {
      k_cfl<Sys, N>(w.data(), g, T, wprod.data(), &st);
    });
    dt_dev(&st);
    {
      StripPlan plan;
      const int cpb = stiff ? NewtonCfg<Sys, N>::CPB : PredCfg<Sys, N>::CPB;
      plan_strips(faces ? g_strips : 1, ndim, g.nX, g.nXw, g.Cw, cpb, N,
                  fi.off, &plan);
      for (int i = 0; i < plan.S; i++) {
        predictor_stage<Sys, N>(stiff != 0, w.data(), qh.data(), g, T,
                                wprod.data(), &st, tol, mixed, 0, plan.blk[i],
                                plan.blk[i + 1]);
        FaceSpan sp;
        long long np = 0;
        for (int d = 0; d < 3; d++) {
          sp.lo[d] = plan.lo[i][d];
          sp.n[d] = plan.n[i][d];
          np += sp.n[d];
        }
        if (faces && np > 0 && FLUX == 0 && FaceSplit<Sys>::OK) {
          // two launches per chunk through the records, as enqueue_faces;
          // a small odd chunk makes chunks straddle the directions
          const long long ch = 61;
          std::vector<double> rec((size_t)FaceSplit<Sys>::REC * ch);
          for (long long q0 = 0; q0 < np; q0 += ch) {
            const long long m = np - q0 < ch ? np - q0 : ch;
            emu::launch(grid_for(m, 128, 152 * 256), 128, 0, [&] {
              k_faces_pre<Sys, N>(qh.data(), rec.data(), ch, g, T, fi, &st,
                                  sp, q0);
            });
            emu::launch(grid_for(m, 128, 152 * 256), 128, 0, [&] {
              k_faces_eig<Sys, N>(rec.data(), ch, contrib.data(), fi, &st,
                                  sp, q0);
            });
          }
        } else if (faces && np > 0) {
          emu::launch(grid_for(np, 128, 152 * 256), 128, 0, [&] {
            k_faces<Sys, N, FLUX>(qh.data(), contrib.data(), g, T, fi, &st,
                                  sp);
          });
        }
      }
    }
    if (centers)
      emu::launch(grid_for(g.C * N * Nd, 128, 152 * 256), 128, 0, [&] {
        k_centers<Sys, N>(qh.data(), cen.data(), g, T, &st);
      });
    emu::launch(grid_for(g.C * V, 256, 152 * 64), 256, 0, [&] {
      k_gather<Sys, N>(u, cen.data(), contrib.data(), g, fi, centers ? 1 : 0,
                       faces ? 1 : 0, &st);
    });
    step_end_dev(&st, 1);
  }
  *t_out = st.t;
  *iters_out = st.pred_iters;
  return st.count;
}

// The predictor stage alone on given reconstruction data w (nrows = cells
// x N^ndim rows), as stage_predictor sets it up; with guess non-null the
// stiff predictor starts from it (the given initial guess of
// stage_predictor).
template <class Sys, int N>
void predictor_only(int ndim, int stiff, const double *w, long long nrows,
                    const double *dX, double dt, double tol, const double *tabs,
                    double *qh, unsigned long long *iters, int *max_iters,
                    int *fail, const double *guess = nullptr,
                    unsigned long long *fallbacks = nullptr, int mixed = 0,
                    unsigned long long *iters32 = nullptr) {
  const Tables T = unpack_tables(N, tabs);
  const int ones[3] = {1, 1, 1};
  Geom g = make_geom(ndim, ones, nullptr, dX, N);
  g.Cw = nrows / ipow(N, ndim);
  const std::vector<double> wprod = make_wprod(T, ndim);
  DevState st;
  std::memset(&st, 0, sizeof(st));
  st.active = 1;
  st.tf = 1;
  st.cfl = 1;
  st.dt = dt;
  st.max_steps = -1;
  st.snap_slot = -1;
  if (guess)
    std::memcpy(qh, guess, sizeof(double) * nrows * N * Sys::V);
  predictor_stage<Sys, N>(stiff != 0, w, qh, g, T, wprod.data(), &st, tol, mixed,
                          guess ? 1 : 0);
  *iters = st.pred_iters;
  *max_iters = st.pred_max_iters;
  *fail = st.pred_fail;
  if (fallbacks)
    *fallbacks = st.pred_fallbacks;
  if (iters32)
    *iters32 = st.pred_iters32;
}
} // namespace

// The (system, ndim, order, flux) combinations this unit instantiates:
// with HOST_USER_SYSTEM (a file holding the `struct UserSystem` that
// pypde_gb300.translate makes from Python callbacks, as the run-time
// compiled kernels include it) and HOST_USER_N, that system under the name
// "user" at order HOST_USER_N with each flux; otherwise the built-ins.
#ifdef HOST_USER_SYSTEM
#include HOST_USER_SYSTEM
#define HOST_CASES(X)                                                          \
  X("user", UserSystem::NDIM, UserSystem, HOST_USER_N, 0)                      \
  X("user", UserSystem::NDIM, UserSystem, HOST_USER_N, 1)                      \
  X("user", UserSystem::NDIM, UserSystem, HOST_USER_N, 2)
#else
#define HOST_CASES(X)                                                          \
  X("euler", 1, Euler<1>, 1, 0)                                                \
  X("euler", 1, Euler<1>, 2, 0)                                                \
  X("euler", 1, Euler<1>, 3, 0)                                                \
  X("euler", 1, Euler<1>, 2, 1)                                                \
  X("euler", 1, Euler<1>, 2, 2)                                                \
  X("euler", 2, Euler<2>, 2, 0)                                                \
  X("euler", 2, Euler<2>, 3, 0)                                                \
  X("euler", 2, Euler<2>, 2, 1)                                                \
  X("euler", 2, Euler<2>, 2, 2)                                                \
  X("euler", 3, Euler<3>, 2, 0)                                                \
  X("cattaneo", 2, Cattaneo<2>, 1, 0)                                          \
  X("cattaneo", 2, Cattaneo<2>, 2, 0)                                          \
  X("cattaneo", 2, Cattaneo<2>, 2, 1)                                          \
  X("cattaneo", 2, Cattaneo<2>, 3, 0)                                          \
  X("cattaneo", 3, Cattaneo<3>, 2, 0)                                          \
  X("ncp", 1, Ncp<1>, 2, 0)                                                    \
  X("ncp", 2, Ncp<2>, 2, 0)                                                    \
  X("ncp", 2, Ncp<2>, 2, 2)                                                    \
  X("burgers2", 1, Burgers2, 3, 0)
#endif

// Fibers run in reverse thread order when reverse is non-zero.
HOST_API void host_set_order(int reverse) { emu::g_reverse = reverse != 0; }

// Predictor strips of the following host_run calls (1 to 32).
HOST_API void host_set_strips(int strips) { g_strips = strips; }

// The strip plan of a grid: returns the strips S and fills blk[0..S] and
// lo/n[s*3 + d] (the arrays hold MAX_STRIPS + 1 and 3 MAX_STRIPS entries).
HOST_API int host_plan_strips(int S, int ndim, const int *nX, int N, int cpb,
                              long long *blk, long long *lo, long long *n) {
  const int ones[3] = {1, 1, 1};
  const double dX[3] = {1, 1, 1};
  const Geom g = make_geom(ndim, nX, ones, dX, N);
  const FaceIndex fi = make_face_index(g, N);
  StripPlan p;
  plan_strips(S, ndim, g.nX, g.nXw, g.Cw, cpb, N, fi.off, &p);
  for (int s = 0; s <= p.S; s++)
    blk[s] = p.blk[s];
  for (int s = 0; s < p.S; s++)
    for (int d = 0; d < 3; d++) {
      lo[s * 3 + d] = p.lo[s][d];
      n[s * 3 + d] = p.n[s][d];
    }
  return p.S;
}

// K steps of a built-in system through the device kernels; returns the
// steps taken, -1 for a combination this unit does not instantiate, or -2
// when a block deadlocked at its barriers.
HOST_API long long host_run(const char *name, int ndim, int N, int flux,
                              double *u, const int *nX, const int *bt,
                              const double *dX, const double *tabs, double tf,
                              double cfl, int stiff, double tol, int mixed,
                              long long max_steps, double *t_out,
                              unsigned long long *iters_out) {
  emu::g_deadlock = false;
#define RUN_CASE(NAME, NDIM, SYS, ORD, FL)                                     \
  if (!std::strcmp(name, NAME) && ndim == NDIM && N == ORD && flux == FL) {    \
    const long long k = run_steps<SYS, ORD, FL>(                               \
        u, ndim, nX, bt, dX, tabs, tf, cfl, stiff, tol, mixed, max_steps,      \
        t_out, iters_out);                                                     \
    return emu::g_deadlock ? -2 : k;                                           \
  }
  HOST_CASES(RUN_CASE)
#undef RUN_CASE
  return -1;
}

// The predictor stage alone; 0, -1 for an unknown combination, or -2 when
// a block deadlocked at its barriers.
HOST_API int host_predictor(const char *name, int ndim, int N, int stiff,
                              const double *w, long long nrows,
                              const double *dX, double dt, double tol,
                              const double *tabs, double *qh,
                              unsigned long long *iters, int *max_iters,
                              int *fail) {
  emu::g_deadlock = false;
#define PRED_CASE(NAME, NDIM, SYS, ORD, FL)                                    \
  if (FL == 0 && !std::strcmp(name, NAME) && ndim == NDIM && N == ORD) {       \
    predictor_only<SYS, ORD>(ndim, stiff, w, nrows, dX, dt, tol, tabs, qh,     \
                             iters, max_iters, fail);                          \
    return emu::g_deadlock ? -2 : 0;                                           \
  }
  HOST_CASES(PRED_CASE)
#undef PRED_CASE
  return -1;
}

namespace {
// Batched steps of problems of one system and order, as run_batch enqueues
// them (enqueue_batch_step): every stage is one launch over all problems
// whose blocks drain a queue of tiles, tile = one block of the stage's
// one-problem launch.  per_pop = 0 launches one block per tile; otherwise
// `ctas` persistent blocks pop per_pop tiles at a time.
enum { B_BND, B_W0, B_W1, B_W2, B_CFL, B_PRED, B_FACES, B_CEN, B_GATHER, B_N };

template <class Sys, int N, int FLUX>
void run_batch_steps(int np, double *u_all, int ndim, const int *nX_all,
                     const int *bt_all, const double *dX_all,
                     const double *tf_all, const double *cfl_all,
                     const double *tabs, int stiff, double tol, int per_pop,
                     int ctas, long long max_steps, long long *steps_out,
                     double *t_out) {
  constexpr int V = Sys::V;
  const Tables T = unpack_tables(N, tabs);
  const int Nd = ipow(N, ndim), NT = N * Nd;
  const bool faces = Sys::HAS_F || Sys::HAS_B;
  const bool centers = Sys::HAS_B || Sys::HAS_S;
  const std::vector<double> wprod = make_wprod(T, ndim);
  std::vector<BatchProblem> P(np);
  std::vector<DevState> S(np);
  std::vector<std::vector<double>> bufs;
  auto buf = [&](long long n) {
    bufs.emplace_back(n > 0 ? n : 1);
    return bufs.back().data();
  };
  std::vector<long long> off[B_N];
  for (int st = 0; st < B_N; st++)
    off[st].push_back(0);
  long long uoff = 0;
  for (int p = 0; p < np; p++) {
    BatchProblem &b = P[p];
    std::memset(&b, 0, sizeof(b));
    b.g = make_geom(ndim, nX_all + p * ndim, bt_all + p * ndim,
                    dX_all + p * ndim, N);
    b.fi = make_face_index(b.g, N);
    b.N = N;
    b.V = V;
    b.u = u_all + uoff;
    uoff += b.g.C * V;
    b.ub = buf(b.g.Cb * V);
    b.w = buf(b.g.Cw * Nd * V);
    b.qh = buf(b.g.Cw * N * Nd * V);
    b.contrib = buf((faces ? b.fi.off[ndim] : 1) * 2 * V);
    b.cen = buf((centers ? b.g.C * NT : 1) * V);
    b.wprod = const_cast<double *>(wprod.data());
    // records of the two-launch faces, as run_batch carves them
    if constexpr (FLUX == 0 && FaceSplit<Sys>::OK)
      b.rec = buf(b.fi.off[ndim] * FaceSplit<Sys>::REC);
    long long tw[3] = {0, 0, 0};
    int m[3] = {b.g.nXb[0], b.g.nXb[1], b.g.nXb[2]};
    const double *src = b.ub;
    int n4 = 1;
    for (int d = 0; d < ndim; d++) {
      long long n1 = 1, n3 = 1;
      for (int e = 0; e < d; e++)
        n1 *= m[e];
      for (int e = d + 1; e < ndim; e++)
        n3 *= m[e];
      tw[d] = n1 * (m[d] - 2 * (N - 1)) * n3 * (long long)n4 * V;
      // each work item writes the N nodal values of one 1-D reconstruction
      double *dst = (d == ndim - 1) ? b.w : buf(tw[d] * N);
      b.win[d] = src;
      b.wout[d] = dst;
      b.wn1[d] = n1;
      b.wn3[d] = n3;
      b.wmd[d] = m[d];
      b.wn4[d] = n4;
      src = dst;
      m[d] -= 2 * (N - 1);
      n4 *= N;
    }
    auto tiles = [](long long work, int per) { return (work + per - 1) / per; };
    long long tl[B_N] = {};
    tl[B_BND] = tiles(b.g.Cb * V, 256);
    for (int d = 0; d < ndim; d++)
      tl[B_W0 + d] = tiles(tw[d], 128);
    tl[B_CFL] = tiles(b.g.Cw, 128);
    tl[B_PRED] = tiles(b.g.Cw, stiff ? NewtonCfg<Sys, N>::CPB
                                     : PredCfg<Sys, N>::CPB);
    tl[B_FACES] = faces ? tiles(b.fi.off[ndim], 128) : 0;
    tl[B_CEN] = centers ? tiles(b.g.C * NT, 128) : 0;
    tl[B_GATHER] = tiles(b.g.C * V, 256);
    for (int st = 0; st < B_N; st++)
      off[st].push_back(off[st].back() + tl[st]);
    DevState &d0 = S[p];
    std::memset(&d0, 0, sizeof(d0));
    d0.tf = tf_all[p];
    d0.cfl = cfl_all[p];
    d0.max_steps = max_steps > 0 ? max_steps : -1;
    d0.ndt = 1;
    d0.snap_slot = -1;
    b.st = &d0;
  }
  unsigned long long heads[B_N];
  auto stage = [&](int st, unsigned threads, size_t smem,
                   const std::function<void(TileQueue, int)> &k) {
    const long long total = off[st].back();
    if (total == 0)
      return;
    heads[st] = 0;
    TileQueue q{off[st].data(), np, &heads[st]};
    unsigned grid;
    if (per_pop == 0) {
      grid = (unsigned)total;
    } else {
      const long long want = (total + per_pop - 1) / per_pop;
      grid = (unsigned)(want < ctas ? want : ctas);
    }
    emu::launch(grid, threads, smem, [&] { k(q, per_pop); });
  };
  const BatchProblem *dP = P.data();
  for (;;) {
    int any = 0;
    for (int p = 0; p < np; p++) {
      step_begin_dev(P[p].st);
      any |= P[p].st->active;
    }
    if (!any || emu::g_deadlock)
      break;
    stage(B_BND, 256, 0, [&](TileQueue q, int pp) { kb_boundaries(dP, q, pp); });
    for (int d = 0; d < ndim; d++)
      stage(B_W0 + d, 128, 0,
            [&](TileQueue q, int pp) { kb_weno<N>(dP, q, pp, d, T); });
    stage(B_CFL, 128, 0,
          [&](TileQueue q, int pp) { kb_cfl<Sys, N>(dP, q, pp, T); });
    for (int p = 0; p < np; p++)
      dt_dev(P[p].st);
    if (stiff)
      stage(B_PRED, NewtonCfg<Sys, N>::THREADS, NewtonCfg<Sys, N>::SMEM_BYTES,
            [&](TileQueue q, int pp) { kb_newton<Sys, N>(dP, q, pp, T, tol, 0); });
    else
      stage(B_PRED, PredCfg<Sys, N>::THREADS,
            (size_t)PredCfg<Sys, N>::SMEM_DOUBLES * 8,
            [&](TileQueue q, int pp) { kb_predictor<Sys, N>(dP, q, pp, T); });
    if (faces && FLUX == 0 && FaceSplit<Sys>::OK) { // two launches, own queues
      stage(B_FACES, 128, 0,
            [&](TileQueue q, int pp) { kb_faces_pre<Sys, N>(dP, q, pp, T); });
      stage(B_FACES, 128, 0,
            [&](TileQueue q, int pp) { kb_faces_eig<Sys, N>(dP, q, pp); });
    } else if (faces) {
      stage(B_FACES, 128, 0,
            [&](TileQueue q, int pp) { kb_faces<Sys, N, FLUX>(dP, q, pp, T); });
    }
    if (centers)
      stage(B_CEN, 128, 0,
            [&](TileQueue q, int pp) { kb_centers<Sys, N>(dP, q, pp, T); });
    stage(B_GATHER, 256, 0, [&](TileQueue q, int pp) {
      kb_gather<Sys, N>(dP, q, pp, centers ? 1 : 0, faces ? 1 : 0);
    });
    for (int p = 0; p < np; p++)
      step_end_dev(P[p].st, 1);
  }
  for (int p = 0; p < np; p++) {
    steps_out[p] = S[p].count;
    t_out[p] = S[p].t;
  }
}
} // namespace

// The stiff predictor started from a given guess (nrows x N rows of V),
// with FP32 sweeps first when mixed is non-zero: qh, iteration counts, the
// cells that fell back to the plain guess and the FP32 sweeps;
// 0, -1 for an unknown combination, or -2 when a block deadlocked.
HOST_API int host_predictor_guess(const char *name, int ndim, int N,
                                    const double *w, long long nrows,
                                    const double *dX, double dt, double tol,
                                    const double *tabs, const double *guess,
                                    double *qh, unsigned long long *iters,
                                    int *max_iters,
                                    unsigned long long *fallbacks, int mixed,
                                    unsigned long long *iters32) {
  emu::g_deadlock = false;
  int fail = 0;
#define GUESS_CASE(NAME, NDIM, SYS, ORD, FL)                                   \
  if (FL == 0 && SYS::HAS_S && !std::strcmp(name, NAME) && ndim == NDIM &&     \
      N == ORD) {                                                              \
    predictor_only<SYS, ORD>(ndim, 1, w, nrows, dX, dt, tol, tabs, qh, iters,  \
                             max_iters, &fail, guess, fallbacks,               \
                             SYS::HAS_FP32 ? mixed : 0, iters32);              \
    return emu::g_deadlock ? -2 : 0;                                           \
  }
  HOST_CASES(GUESS_CASE)
#undef GUESS_CASE
  return -1;
}

// The mixed-precision stiff predictor alone (FP32 sweeps, then FP64): qh,
// FP64 iterations, their per-cell maximum and the FP32 sweeps; 0, -1 for an
// unknown combination, or -2 when a block deadlocked.
HOST_API int host_predictor_mixed(const char *name, int ndim, int N,
                                  const double *w, long long nrows,
                                  const double *dX, double dt, double tol,
                                  const double *tabs, double *qh,
                                  unsigned long long *iters, int *max_iters,
                                  unsigned long long *iters32) {
  emu::g_deadlock = false;
  int fail = 0;
#define MIXED_CASE(NAME, NDIM, SYS, ORD, FL)                                   \
  if (FL == 0 && SYS::HAS_FP32 && !std::strcmp(name, NAME) && ndim == NDIM &&  \
      N == ORD) {                                                              \
    predictor_only<SYS, ORD>(ndim, 1, w, nrows, dX, dt, tol, tabs, qh, iters,  \
                             max_iters, &fail, nullptr, nullptr, 1, iters32);  \
    return emu::g_deadlock ? -2 : 0;                                           \
  }
  HOST_CASES(MIXED_CASE)
#undef MIXED_CASE
  return -1;
}

// np problems of one built-in system and order stepped as one batch; u_all
// holds their states one after the other, nX/bt/dX are np x ndim.  0, -1
// for an unknown combination, or -2 when a block deadlocked.
HOST_API int host_run_batch(const char *name, int ndim, int N, int flux,
                              int np, double *u_all, const int *nX,
                              const int *bt, const double *dX,
                              const double *tf, const double *cfl,
                              const double *tabs, int stiff, double tol,
                              int per_pop, int ctas, long long max_steps,
                              long long *steps_out, double *t_out) {
  emu::g_deadlock = false;
#define BATCH_CASE(NAME, NDIM, SYS, ORD, FL)                                   \
  if (!std::strcmp(name, NAME) && ndim == NDIM && N == ORD && flux == FL) {    \
    run_batch_steps<SYS, ORD, FL>(np, u_all, ndim, nX, bt, dX, tf, cfl, tabs,  \
                                  stiff, tol, per_pop, ctas, max_steps,        \
                                  steps_out, t_out);                           \
    return emu::g_deadlock ? -2 : 0;                                           \
  }
  HOST_CASES(BATCH_CASE)
#undef BATCH_CASE
  return -1;
}
