// runtime.cu -- host driver of the ADER-WENO step on one GPU.
//
// Replaces the reference's time loop and thread pool
// (haranjackson/PyPDE src/solvers/iterator.cpp:38-151,
// include/ThreadPool.h): the whole grid is resident in HBM, every stage is
// a kernel, and runs of steps are captured in one CUDA graph so the host
// only synchronises between graph launches (to drain snapshots and to see
// whether t reached tf; kernels of steps past the end return at once).
#include "runtime.h"
#include "strips.h"
#include "step_kernels.cuh"
#include "../../include/pypde_gb300.h"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace pypde {

// NVTX ranges name a run and, when the stages are launched one by one
// (profile mode), each stage, so a profiler can select a stage's kernels
// (ncu --nvtx --nvtx-include).  Without a profiler attached they cost a
// branch.  Stages: pop the previous range and push the next.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};
struct NvtxStages {
  bool open = false;
  void next(const char *name) {
    if (open)
      nvtxRangePop();
    nvtxRangePushA(name);
    open = true;
  }
  ~NvtxStages() {
    if (open)
      nvtxRangePop();
  }
};

static thread_local std::string g_err;
void set_error(const std::string &m) { g_err = m; }
const char *last_error() { return g_err.c_str(); }

#define CK(x)                                                                  \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) {                                                   \
      set_error(std::string(#x) + ": " + cudaGetErrorString(e_));             \
      return PYPDE_ERR_CUDA;                                                   \
    }                                                                          \
  } while (0)

// ------------------------------------------------------------------
// registry of built-in systems
// ------------------------------------------------------------------
static std::vector<SystemDesc> &builtins() {
  static std::vector<SystemDesc> v;
  return v;
}
// Each instantiation unit registers one (system, order); the orders of a
// system are merged into one description.
void register_builtin(const SystemDesc &d) {
  for (auto &e : builtins())
    if (e.name == d.name && e.ndim == d.ndim) {
      for (int n = 0; n <= MAXN; n++)
        if (d.have[n]) {
          e.sets[n] = d.sets[n];
          e.have[n] = true;
        }
      return;
    }
  builtins().push_back(d);
}
const SystemDesc *find_builtin(const std::string &name, int ndim) {
  for (auto &d : builtins())
    if (d.name == name && d.ndim == ndim)
      return &d;
  return nullptr;
}

// ------------------------------------------------------------------
// launching AOT or run-time compiled kernels
// ------------------------------------------------------------------
typedef int (*cuLaunchKernel_t)(void *, unsigned, unsigned, unsigned,
                                unsigned, unsigned, unsigned, unsigned,
                                cudaStream_t, void **, void **);
static cuLaunchKernel_t driver_launch() {
  static cuLaunchKernel_t fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuLaunchKernel", &p, 12000,
                                         cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (cuLaunchKernel_t)p;
  }
  return fn;
}

static cudaError_t launch(const KFunc &f, dim3 grid, dim3 block, size_t smem,
                          cudaStream_t s, void **args) {
  if (f.aot)
    return cudaLaunchKernel(f.aot, grid, block, args, smem, s);
  cuLaunchKernel_t fn = driver_launch();
  if (!fn || !f.jit)
    return cudaErrorInvalidDeviceFunction;
  int r = fn(f.jit, grid.x, grid.y, grid.z, block.x, block.y, block.z,
             (unsigned)smem, s, args, nullptr);
  return r == 0 ? cudaSuccess : cudaErrorLaunchFailure;
}

// Opts the kernel in to `bytes` of dynamic shared memory.  Set whenever the
// kernel uses any: the 48 KB default covers static plus dynamic shared
// memory, and the static part is only known after the device link.
static cudaError_t set_smem(const KFunc &f, size_t bytes) {
  if (bytes == 0)
    return cudaSuccess;
  if (f.aot)
    return cudaFuncSetAttribute(f.aot,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)bytes);
  typedef int (*cuFuncSetAttribute_t)(void *, int, int);
  void *p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuFuncSetAttribute", &p, 12000,
                                       cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return cudaErrorInvalidDeviceFunction;
  // CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES = 8
  return ((cuFuncSetAttribute_t)p)(f.jit, 8, (int)bytes) == 0
             ? cudaSuccess
             : cudaErrorInvalidValue;
}

static unsigned grid_for(long long work, int threads, int cap_blocks) {
  long long b = (work + threads - 1) / threads;
  if (b < 1)
    b = 1;
  if (b > cap_blocks)
    b = cap_blocks;
  return (unsigned)b;
}

// ------------------------------------------------------------------
// device memory: grow-only buffers per device, reused across calls
// ------------------------------------------------------------------
struct Buf {
  void *p = nullptr;
  size_t cap = 0;
};
static cudaError_t ensure(Buf &b, size_t bytes) {
  if (bytes == 0)
    bytes = 8;
  if (b.cap >= bytes)
    return cudaSuccess;
  if (b.p)
    cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e == cudaSuccess)
    b.cap = bytes;
  return e;
}
struct Arena {
  Buf u, uprev, ub, tmpA, tmpB, w, qh, contrib, cen, ring, state, wprod;
  Buf facerec; // records between k_faces_pre and k_faces_eig
  DevState *host_state = nullptr; // pinned
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;    // faces of finished predictor strips
  cudaEvent_t strip_ev[MAX_STRIPS + 1] = {};
};
static std::mutex g_mu;
static std::map<int, Arena> g_arena;

static int arena_for(int device, Arena **out) {
  int n = 0;
  CK(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) {
    set_error("invalid CUDA device ordinal");
    return PYPDE_ERR_ARG;
  }
  CK(cudaSetDevice(device));
  Arena &a = g_arena[device];
  if (!a.stream)
    CK(cudaStreamCreateWithFlags(&a.stream, cudaStreamNonBlocking));
  if (!a.side) {
    CK(cudaStreamCreateWithFlags(&a.side, cudaStreamNonBlocking));
    for (int i = 0; i <= MAX_STRIPS; i++)
      CK(cudaEventCreateWithFlags(&a.strip_ev[i], cudaEventDisableTiming));
  }
  if (!a.host_state)
    CK(cudaMallocHost(&a.host_state, sizeof(DevState)));
  *out = &a;
  return PYPDE_OK;
}

// ------------------------------------------------------------------
// geometry
// ------------------------------------------------------------------
static void fill_geom(Geom &g, int ndim, const int *nX, const int *bt,
                      const double *dX, int N) {
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
}

static FaceIndex face_index(const Geom &g, int N) {
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

static int ipow(int b, int e) {
  int r = 1;
  while (e-- > 0)
    r *= b;
  return r;
}

// ------------------------------------------------------------------
// WENO passes (generic in V, templated on N)
// ------------------------------------------------------------------
static const void *weno_kernel(int N) {
  switch (N) {
  case 1: return (const void *)&k_weno_pass<1>;
  case 2: return (const void *)&k_weno_pass<2>;
  case 3: return (const void *)&k_weno_pass<3>;
  case 4: return (const void *)&k_weno_pass<4>;
  case 5: return (const void *)&k_weno_pass<5>;
  case 6: return (const void *)&k_weno_pass<6>;
  default: return nullptr;
  }
}

// Enqueue the ndim passes: in has shape m (ndim dims) with one node per
// cell; the last pass writes w.  tmpA/tmpB hold intermediate passes.
static cudaError_t enqueue_weno(const double *in, const int *m_in, int ndim,
                                int N, int V, const Tables &T, double *tmpA,
                                double *tmpB, double *w, const DevState *st,
                                cudaStream_t s) {
  const void *fn = weno_kernel(N);
  if (!fn)
    return cudaErrorInvalidValue;
  int m[3];
  for (int d = 0; d < ndim; d++)
    m[d] = m_in[d];
  const double *src = in;
  int n4 = 1;
  for (int d = 0; d < ndim; d++) {
    long long n1 = 1, n3 = 1;
    for (int e = 0; e < d; e++)
      n1 *= m[e];
    for (int e = d + 1; e < ndim; e++)
      n3 *= m[e];
    int md = m[d];
    double *dst = (d == ndim - 1) ? w : ((d % 2 == 0) ? tmpA : tmpB);
    long long total = n1 * (md - 2 * (N - 1)) * n3 * (long long)n4 * V;
    Tables Tc = T;
    void *args[] = {(void *)&src, (void *)&dst, (void *)&n1, (void *)&md,
                    (void *)&n3,  (void *)&n4,  (void *)&V,  (void *)&Tc,
                    (void *)&st};
    cudaError_t e = cudaLaunchKernel(fn, dim3(grid_for(total, 128, 152 * 64)),
                                     dim3(128), args, 0, s);
    if (e != cudaSuccess)
      return e;
    src = dst;
    m[d] -= 2 * (N - 1);
    n4 *= N;
  }
  return cudaSuccess;
}

static long long weno_tmp_doubles(const int *nXb, int ndim, int N, int V) {
  // largest intermediate pass output (all but the last)
  long long best = 0;
  int m[3];
  for (int d = 0; d < ndim; d++)
    m[d] = nXb[d];
  long long n4 = 1;
  for (int d = 0; d < ndim - 1; d++) {
    m[d] -= 2 * (N - 1);
    n4 *= N;
    long long sz = n4 * V;
    for (int e = 0; e < ndim; e++)
      sz *= m[e];
    if (sz > best)
      best = sz;
  }
  return best;
}

// ------------------------------------------------------------------
// one step, enqueued on a stream (captured into the graph)
// ------------------------------------------------------------------
struct StepCtx {
  const SystemDesc *sys;
  const KernelSet *ks;
  Geom g;
  FaceIndex fi;
  Tables T;
  int N, V, ring, flux;
  double tol;
  bool stiff, faces, centers;
  double *u, *uprev, *ub, *tmpA, *tmpB, *w, *qh, *contrib, *cen, *ringbuf,
      *wprod;
  DevState *st;
  const WarmStart *warm; // learned warm start of the Newton predictor
  int mixed;             // FP32 Newton sweeps first (mixed precision)
  const double *guess;   // or a given initial guess already in qh
  // harvest of training pairs (device buffers)
  double *hw, *hq, *hdt;
  long long hstride, hper;
  int hsteps;
  // predictor strips overlapped with the faces (null: one launch each)
  const StripPlan *plan;
  cudaStream_t side;
  cudaEvent_t *strip_ev;
  // Rusanov faces in two launches, face_ch points at a time (null: one)
  double *facerec;
  long long face_ch;
};

// Face points per k_faces_pre / k_faces_eig pair: the record buffer holds
// this many (73 doubles each for the 2-D relaxation system: 2.4 GB).
constexpr long long FACE_CHUNK = 1LL << 22;

// Whether a step runs its predictor in strips with the faces of finished
// strips on the side stream (not in the stage-timing mode, whose events
// bracket one stage at a time).
static bool overlapped(const StepCtx &c, bool profile) {
  return !profile && c.plan && c.plan->S > 1 && c.faces;
}

static FaceSpan whole_span(const StepCtx &c) {
  FaceSpan sp;
  for (int d = 0; d < 3; d++) {
    sp.lo[d] = d < c.g.ndim ? c.fi.off[d] : 0;
    sp.n[d] = d < c.g.ndim ? c.fi.off[d + 1] - c.fi.off[d] : 0;
  }
  return sp;
}

static FaceSpan strip_span(const StripPlan &p, int i) {
  FaceSpan sp;
  for (int d = 0; d < 3; d++) {
    sp.lo[d] = p.lo[i][d];
    sp.n[d] = p.n[i][d];
  }
  return sp;
}

static long long span_points(const FaceSpan &sp) {
  return sp.n[0] + sp.n[1] + sp.n[2];
}

static bool split_faces(const StepCtx &c) {
  return c.flux == 0 && c.facerec && c.ks->face_rec > 0;
}

static cudaError_t enqueue_faces(const StepCtx &c, cudaStream_t s,
                                 const FaceSpan &span) {
  const long long n = span_points(span);
  if (n == 0)
    return cudaSuccess;
  Geom g = c.g;
  Tables T = c.T;
  FaceIndex fi = c.fi;
  FaceSpan sp = span;
  if (split_faces(c)) { // chunks of face_ch points through the records
    long long ch = c.face_ch;
    for (long long q0 = 0; q0 < n; q0 += ch) {
      const long long m = (n - q0 < ch) ? n - q0 : ch;
      const dim3 grid(grid_for(m, 128, 152 * 256));
      void *pa[] = {(void *)&c.qh, (void *)&c.facerec, (void *)&ch,
                    (void *)&g,    (void *)&T,         (void *)&fi,
                    (void *)&c.st, (void *)&sp,        (void *)&q0};
      cudaError_t e = launch(c.ks->faces_pre, grid, dim3(128), 0, s, pa);
      if (e != cudaSuccess)
        return e;
      void *ea[] = {(void *)&c.facerec, (void *)&ch, (void *)&c.contrib,
                    (void *)&fi,        (void *)&c.st, (void *)&sp,
                    (void *)&q0};
      e = launch(c.ks->faces_eig, grid, dim3(128), 0, s, ea);
      if (e != cudaSuccess)
        return e;
    }
    return cudaSuccess;
  }
  void *a[] = {(void *)&c.qh, (void *)&c.contrib, (void *)&g, (void *)&T,
               (void *)&fi,   (void *)&c.st,      (void *)&sp};
  return launch(c.ks->faces_flux[c.flux], dim3(grid_for(n, 128, 152 * 256)),
                dim3(128), 0, s, a);
}

// Launches enqueue_faces makes for a span.
static int face_launches(const StepCtx &c, const FaceSpan &sp) {
  const long long n = span_points(sp);
  if (n == 0)
    return 0;
  return split_faces(c) ? (int)(2 * ((n + c.face_ch - 1) / c.face_ch)) : 1;
}

// The warm-start network's guess of qh (learned form): qh = w + its
// correction, from which the Newton iteration starts.
static cudaError_t enqueue_guess(const StepCtx &c, cudaStream_t s) {
  if (!c.stiff || !c.warm)
    return cudaSuccess;
  const KernelSet &k = *c.ks;
  Geom g = c.g;
  MlpModel m = c.warm->model;
  void *ga[] = {(void *)&c.w, (void *)&c.qh, (void *)&g, (void *)&m,
                (void *)&c.st};
  long long tiles = (g.Cw + 127) / 128;
  unsigned gb = (unsigned)(tiles < 152 * 2 ? tiles : 152 * 2);
  return launch(k.guess, dim3(gb), dim3(256), k.guess_smem, s, ga);
}

static int predictor_cpb(const StepCtx &c) {
  return c.stiff ? c.ks->newton_cpb : c.ks->pred_cpb;
}

// Predictor blocks [b_lo, b_hi): cells [b_lo cpb, b_hi cpb) of the w-grid.
static cudaError_t enqueue_predictor_blocks(const StepCtx &c, cudaStream_t s,
                                            long long b_lo, long long b_hi) {
  if (b_hi <= b_lo)
    return cudaSuccess;
  const KernelSet &k = *c.ks;
  Geom g = c.g;
  Tables T = c.T;
  double tol = c.tol;
  long long b0 = b_lo;
  const dim3 grid((unsigned)(b_hi - b_lo));
  if (c.stiff) {
    int guess = (c.warm || c.guess) ? 1 : 0;
    int mixed = c.mixed;
    void *na[] = {(void *)&c.w,     (void *)&c.qh,    (void *)&g,
                  (void *)&T,       (void *)&c.wprod, (void *)&c.st,
                  (void *)&tol,     (void *)&guess,   (void *)&mixed,
                  (void *)&b0};
    return launch(k.newton, grid, dim3(k.newton_threads), k.newton_smem, s,
                  na);
  }
  void *args[] = {(void *)&c.w,     (void *)&c.qh, (void *)&g, (void *)&T,
                  (void *)&c.wprod, (void *)&c.st, (void *)&b0};
  return launch(k.predictor, grid, dim3(k.pred_threads), k.pred_smem, s,
                args);
}

static cudaError_t enqueue_predictor(const StepCtx &c, cudaStream_t s) {
  cudaError_t e = enqueue_guess(c, s);
  if (e != cudaSuccess)
    return e;
  const int cpb = predictor_cpb(c);
  return enqueue_predictor_blocks(c, s, 0, (c.g.Cw + cpb - 1) / cpb);
}

static cudaError_t enqueue_fv(const StepCtx &c, cudaStream_t s) {
  const KernelSet &k = *c.ks;
  Geom g = c.g;
  Tables T = c.T;
  FaceIndex fi = c.fi;
  cudaError_t e;
  if (c.faces) {
    e = enqueue_faces(c, s, whole_span(c));
    if (e != cudaSuccess)
      return e;
  }
  if (c.centers) {
    long long nn = (long long)c.N * ipow(c.N, c.g.ndim);
    void *a[] = {(void *)&c.qh, (void *)&c.cen, (void *)&g, (void *)&T,
                 (void *)&c.st};
    e = launch(k.centers, dim3(grid_for(g.C * nn, 128, 152 * 256)),
               dim3(128), 0, s, a);
    if (e != cudaSuccess)
      return e;
  }
  int uc = c.centers ? 1 : 0, uf = c.faces ? 1 : 0;
  void *a[] = {(void *)&c.u, (void *)&c.cen, (void *)&c.contrib, (void *)&g,
               (void *)&fi,  (void *)&uc,    (void *)&uf,        (void *)&c.st};
  return launch(k.gather, dim3(grid_for(g.C * c.V, 256, 152 * 64)), dim3(256),
                0, s, a);
}

// Kernels one step launches (the count reported as kernel_launches).
static int kernels_per_step(const StepCtx &c, bool profile) {
  int pred = 1, faces = c.faces ? face_launches(c, whole_span(c)) : 0;
  if (overlapped(c, profile)) {
    pred = faces = 0;
    for (int i = 0; i < c.plan->S; i++) {
      pred += c.plan->blk[i + 1] > c.plan->blk[i];
      faces += face_launches(c, strip_span(*c.plan, i));
    }
  }
  // step begin, copy of u, ghost fill, CFL, dt, gather, step end, snapshot
  return 8 + c.g.ndim + pred + faces + (c.centers ? 1 : 0) +
         (c.stiff && c.warm ? 1 : 0) + (c.hw ? 1 : 0);
}

// One step.  With ev non-null, events are recorded between the stages
// (ev[0..8]: start, after ghost fill, WENO, CFL+dt, predictor, faces,
// centres, gather, end) for the profiling mode.
static cudaError_t enqueue_step(const StepCtx &c, cudaStream_t s,
                                cudaEvent_t *ev = nullptr) {
  cudaError_t e;
  static const char *const kStage[8] = {"ghost fill", "weno",  "cfl+dt",
                                        "predictor",  "faces", "centres",
                                        "gather",     "step end"};
  NvtxStages nv;
  auto mark = [&](int i) {
    if (ev)
      cudaEventRecord(ev[i], s);
    if (i < 8)
      nv.next(kStage[i]);
  };
  k_step_begin<<<1, 1, 0, s>>>(c.st);
  long long n = c.g.C * c.V;
  k_copy_prev<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(c.u, c.uprev, n,
                                                         c.st);
  mark(0);
  k_boundaries<<<grid_for(c.g.Cb * c.V, 256, 152 * 32), 256, 0, s>>>(
      c.u, c.ub, c.g, c.N, c.V, c.st);
  mark(1);
  e = enqueue_weno(c.ub, c.g.nXb, c.g.ndim, c.N, c.V, c.T, c.tmpA, c.tmpB,
                   c.w, c.st, s);
  if (e != cudaSuccess)
    return e;
  mark(2);
  {
    Geom g = c.g;
    Tables T = c.T;
    void *a[] = {(void *)&c.w, (void *)&g, (void *)&T, (void *)&c.wprod,
                 (void *)&c.st};
    e = launch(c.ks->cfl, dim3(grid_for(c.g.Cw, 128, 152 * 64)), dim3(128), 0,
               s, a);
    if (e != cudaSuccess)
      return e;
  }
  k_dt<<<1, 1, 0, s>>>(c.st);
  mark(3);
  const bool strips = overlapped(c, ev != nullptr);
  bool side_used = false;
  if (strips) {
    // strip i of the predictor on s, then the faces it releases on the side
    // stream while strip i+1 is predicted; the two streams write disjoint
    // parts of qh and contrib
    const StripPlan &p = *c.plan;
    e = enqueue_guess(c, s);
    for (int i = 0; i < p.S && e == cudaSuccess; i++) {
      e = enqueue_predictor_blocks(c, s, p.blk[i], p.blk[i + 1]);
      const FaceSpan sp = strip_span(p, i);
      if (e != cudaSuccess || span_points(sp) == 0)
        continue;
      if ((e = cudaEventRecord(c.strip_ev[i], s)) != cudaSuccess ||
          (e = cudaStreamWaitEvent(c.side, c.strip_ev[i], 0)) != cudaSuccess)
        break;
      side_used = true;
      e = enqueue_faces(c, c.side, sp);
    }
  } else {
    e = enqueue_predictor(c, s);
  }
  if (e != cudaSuccess)
    return e;
  if (c.hw) {
    const int Nd = ipow(c.N, c.g.ndim);
    const int nw = Nd * c.V, nq = c.N * Nd * c.V;
    k_harvest<<<grid_for(c.hper * (nw + nq), 256, 152 * 8), 256, 0, s>>>(
        c.w, c.qh, c.g.Cw, nw, nq, c.st, c.hw, c.hq, c.hdt, c.hstride,
        c.hsteps, c.hper);
  }
  mark(4);
  if (c.faces && !strips) {
    e = enqueue_faces(c, s, whole_span(c));
    if (e != cudaSuccess)
      return e;
  }
  mark(5);
  if (c.centers) {
    // with strips, beside the last faces
    long long nn = (long long)c.N * ipow(c.N, c.g.ndim);
    Geom g = c.g;
    Tables T = c.T;
    void *a[] = {(void *)&c.qh, (void *)&c.cen, (void *)&g, (void *)&T,
                 (void *)&c.st};
    e = launch(c.ks->centers, dim3(grid_for(g.C * nn, 128, 152 * 256)),
               dim3(128), 0, s, a);
    if (e != cudaSuccess)
      return e;
  }
  mark(6);
  if (side_used) { // the gather reads every face's contribution
    if ((e = cudaEventRecord(c.strip_ev[MAX_STRIPS], c.side)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(s, c.strip_ev[MAX_STRIPS], 0)) != cudaSuccess)
      return e;
  }
  {
    Geom g = c.g;
    FaceIndex fi = c.fi;
    int uc = c.centers ? 1 : 0, uf = c.faces ? 1 : 0;
    void *a[] = {(void *)&c.u, (void *)&c.cen, (void *)&c.contrib,
                 (void *)&g,   (void *)&fi,    (void *)&uc,
                 (void *)&uf,  (void *)&c.st};
    e = launch(c.ks->gather, dim3(grid_for(g.C * c.V, 256, 152 * 64)),
               dim3(256), 0, s, a);
    if (e != cudaSuccess)
      return e;
  }
  mark(7);
  k_step_end<<<1, 1, 0, s>>>(c.st, c.ring);
  k_snapshot<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(c.u, c.ringbuf, n,
                                                        c.st);
  mark(8);
  return cudaGetLastError();
}

// A periodic axis wraps ghost cells around once (boundaries.cpp:7-23), which
// needs at least N cells on it; a transmissive axis has no such limit.
static int check_grid(int ndim, const int *nX, const int *bt, int N) {
  for (int d = 0; d < ndim; d++) {
    if (nX[d] < 1) {
      set_error("grid sizes must be positive");
      return PYPDE_ERR_ARG;
    }
    // the ghost fill treats every non-zero type as periodic
    if (bt && bt[d] != 0 && bt[d] != 1) {
      set_error("boundaryTypes must be 0 (transmissive) or 1 (periodic)");
      return PYPDE_ERR_ARG;
    }
    if (bt && bt[d] == 1 && nX[d] < N) {
      set_error("a periodic axis needs at least N cells (axis " +
                std::to_string(d) + " has " + std::to_string(nX[d]) + ")");
      return PYPDE_ERR_ARG;
    }
  }
  return PYPDE_OK;
}

int jit_ensure(SystemDesc &d, int N);

// Kernels of a run-time compiled system are built on first use of an order
// N, on the current device (called after the device is selected).
static int ensure_kernels(const SystemDesc &sys, int N) {
  if (N < 1 || N > MAXN || sys.have[N] || !sys.module)
    return PYPDE_OK;
  return jit_ensure(const_cast<SystemDesc &>(sys), N);
}

static int check_system(const SystemDesc &sys, int ndim, int N, bool stiff,
                        int flux) {
  if (sys.ndim != ndim) {
    set_error("system was built for another number of dimensions");
    return PYPDE_ERR_ARG;
  }
  // checked for every system: faces_flux[flux] is indexed at launch
  if (flux < 0 || flux > 2) {
    set_error("FLUX must be 0 (Rusanov), 1 (Roe) or 2 (Osher)");
    return PYPDE_ERR_ARG;
  }
  if (sys.module && N >= 1 && N <= 3)
    return PYPDE_OK; // compiled on first use (ensure_kernels)
  if (N < 1 || N > MAXN || !sys.have[N]) {
    set_error("order N=" + std::to_string(N) + " is not built for system " +
              sys.name);
    return PYPDE_ERR_UNSUPPORTED;
  }
  if (stiff && !sys.sets[N].newton.valid()) {
    set_error("stiff predictor not built for system " + sys.name);
    return PYPDE_ERR_UNSUPPORTED;
  }
  if (!sys.sets[N].faces_flux[flux].valid()) {
    set_error("flux " + std::to_string(flux) + " is not built for system " +
              sys.name);
    return PYPDE_ERR_UNSUPPORTED;
  }
  return PYPDE_OK;
}

// ------------------------------------------------------------------
// the solver (pde_solver)
// ------------------------------------------------------------------
// Device allocations owned by one call (training-data buffers).
struct DeviceBuffers {
  std::vector<void *> ptrs;
  cudaError_t alloc(void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 8);
    if (e == cudaSuccess)
      ptrs.push_back(*p);
    return e;
  }
  ~DeviceBuffers() {
    for (void *p : ptrs)
      cudaFree(p);
  }
};

// A warm start fits (system, N) when its layer widths are the ones the
// system's guess kernel was built for and it lives on the run's device.
static int check_warm(const SystemDesc &sys, int N, bool stiff, int device,
                      const WarmStart *w) {
  const KernelSet &k = sys.sets[N];
  if (!stiff) {
    set_error("the learned warm start applies to the stiff (Newton) "
              "predictor only");
    return PYPDE_ERR_ARG;
  }
  if (!k.guess.valid() || k.guess_k1 == 0) {
    set_error("no warm-start kernel for system " + sys.name + " at this order");
    return PYPDE_ERR_ARG;
  }
  if (w->model.k1 != k.guess_k1 || w->model.no != k.guess_no ||
      w->model.tau_var >= sys.V || w->device != device) {
    set_error("warm start does not fit system " + sys.name + ": expected k1=" +
              std::to_string(k.guess_k1) + ", no=" +
              std::to_string(k.guess_no) + " on device " +
              std::to_string(device));
    return PYPDE_ERR_ARG;
  }
  return PYPDE_OK;
}

int run_solver(const SystemDesc &sys, const RunArgs &a, Stats *out) {
  NvtxRange nvtx_run("pde_solver");
  if (a.ndim < 1 || a.ndim > 3 || !a.u || a.tf < 0 || a.ndt < 1) {
    set_error("invalid arguments");
    return PYPDE_ERR_ARG;
  }
  for (int d = 0; d < a.ndim; d++)
    if (a.nX[d] < 1 || !(a.dX[d] > 0)) {
      set_error("invalid grid");
      return PYPDE_ERR_ARG;
    }
  int rc = check_system(sys, a.ndim, a.N, a.stiff, a.flux);
  if (rc)
    return rc;
  if ((rc = check_grid(a.ndim, a.nX, a.bt, a.N)))
    return rc;
  if ((a.useF != sys.has_F) || (a.useB != sys.has_B) ||
      (a.useS != sys.has_S)) {
    set_error("useF/useB/useS do not match the callbacks of system " +
              sys.name);
    return PYPDE_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  Arena *ar;
  rc = arena_for(a.device, &ar);
  if (rc)
    return rc;
  if ((rc = ensure_kernels(sys, a.N)))
    return rc;
  if (a.warm && (rc = check_warm(sys, a.N, a.stiff, a.device, a.warm)))
    return rc;
  cudaStream_t s = ar->stream;
  StepCtx c;
  c.sys = &sys;
  c.ks = &sys.sets[a.N];
  c.N = a.N;
  c.V = sys.V;
  fill_geom(c.g, a.ndim, a.nX, a.bt, a.dX, a.N);
  c.fi = face_index(c.g, a.N);
  if (make_tables(a.N, &c.T)) {
    set_error("bad order");
    return PYPDE_ERR_ARG;
  }
  c.stiff = a.stiff;
  c.flux = a.flux;
  c.tol = a.newton_tol;
  c.warm = a.warm;
  c.mixed = a.mixed ? 1 : 0;
  c.guess = nullptr;
  c.hw = c.hq = c.hdt = nullptr;
  c.hstride = 1;
  c.hper = 0;
  c.hsteps = 0;
  c.faces = sys.has_F || sys.has_B;
  c.centers = sys.has_B || sys.has_S;
  StripPlan plan;
  {
    const int cpb = predictor_cpb(c);
    const long long blocks = (c.g.Cw + cpb - 1) / cpb;
    // Automatic: 4 strips for the Newton predictor when each holds at least
    // 4 blocks per SM and the faces run as the one-launch k_faces (255
    // registers, 2 blocks an SM: 1024^2 relaxation with that kernel, 85.0
    // ms a step against 90.0 without strips; 8 strips 85.2, 16 strips
    // 85.5).  The two-launch Rusanov faces fill the SMs themselves (128
    // registers, 4 blocks an SM) and lose with strips (79.3 ms a step
    // without, 83.6 with 4, 83.8 with 2).  The Picard predictor is a small
    // part of its step and gains nothing (512^2 shear layer, N=3: 13.9 ms
    // with 8 strips against 13.65).
    const bool two_launch_faces = c.faces && c.flux == 0 && c.ks->face_rec > 0;
    int S = a.strips;
    if (S == 0)
      S = (c.stiff && !two_launch_faces && blocks >= 4LL * 152 * 4) ? 4 : 1;
    plan_strips(S, a.ndim, c.g.nX, c.g.nXw, c.g.Cw, cpb, c.N, c.fi.off,
                &plan);
  }
  c.plan = &plan;
  c.side = ar->side;
  c.strip_ev = ar->strip_ev;
  c.facerec = nullptr;
  c.face_ch = 0;
  const int V = c.V, N = c.N, Nd = ipow(N, a.ndim);
  long long usz = c.g.C * V;
  int K = a.steps_per_graph;
  if (K <= 0) {
    long long k = (1LL << 21) / (c.g.C * N * Nd);
    K = (int)(k < 1 ? 1 : (k > 32 ? 32 : k));
  }
  c.ring = K + 1;
  CK(ensure(ar->u, usz * 8));
  CK(ensure(ar->uprev, usz * 8));
  CK(ensure(ar->ub, c.g.Cb * V * 8));
  long long tmpn = weno_tmp_doubles(c.g.nXb, a.ndim, N, V);
  CK(ensure(ar->tmpA, tmpn * 8));
  CK(ensure(ar->tmpB, tmpn * 8));
  CK(ensure(ar->w, c.g.Cw * Nd * V * 8));
  CK(ensure(ar->qh, c.g.Cw * N * Nd * V * 8));
  CK(ensure(ar->contrib, (c.faces ? c.fi.off[a.ndim] : 1) * 2 * V * 8));
  CK(ensure(ar->cen, (c.centers ? c.g.C * N * Nd : 1) * V * 8));
  CK(ensure(ar->ring, c.ring * usz * 8));
  if (c.faces && c.flux == 0 && c.ks->face_rec > 0) {
    const long long pts = c.fi.off[a.ndim];
    const long long ch = pts < FACE_CHUNK ? pts : FACE_CHUNK;
    if (ensure(ar->facerec, (long long)c.ks->face_rec * ch * 8) ==
        cudaSuccess) {
      c.face_ch = ch;
      c.facerec = (double *)ar->facerec.p;
    } else { // no room for the records: the faces run as one launch
      cudaGetLastError();
    }
  }
  CK(ensure(ar->state, sizeof(DevState)));
  CK(ensure(ar->wprod, Nd * 8));
  c.u = (double *)ar->u.p;
  c.uprev = (double *)ar->uprev.p;
  c.ub = (double *)ar->ub.p;
  c.tmpA = (double *)ar->tmpA.p;
  c.tmpB = (double *)ar->tmpB.p;
  c.w = (double *)ar->w.p;
  c.qh = (double *)ar->qh.p;
  c.contrib = (double *)ar->contrib.p;
  c.cen = (double *)ar->cen.p;
  c.ringbuf = (double *)ar->ring.p;
  c.wprod = (double *)ar->wprod.p;
  c.st = (DevState *)ar->state.p;
  {
    std::vector<double> wp(Nd);
    make_wprod(c.T, a.ndim, wp.data());
    CK(cudaMemcpyAsync(c.wprod, wp.data(), Nd * 8, cudaMemcpyHostToDevice,
                       s));
  }
  CK(set_smem(c.ks->predictor, c.ks->pred_smem));
  if (c.stiff)
    CK(set_smem(c.ks->newton, c.ks->newton_smem));
  if (c.stiff && c.warm)
    CK(set_smem(c.ks->guess, c.ks->guess_smem));
  DeviceBuffers hbuf; // harvest buffers, freed on every return
  if (a.harvest && a.harvest->steps > 0 && a.harvest->per_step > 0) {
    const HarvestArgs &h = *a.harvest;
    if (!h.w || !h.qh || !h.dt || h.stride < 1) {
      set_error("harvest: missing output arrays or bad stride");
      return PYPDE_ERR_ARG;
    }
    long long rows = (long long)h.steps * h.per_step;
    CK(hbuf.alloc((void **)&c.hw, rows * Nd * V * 8));
    CK(hbuf.alloc((void **)&c.hq, rows * N * Nd * V * 8));
    CK(hbuf.alloc((void **)&c.hdt, h.steps * 8));
    CK(cudaMemsetAsync(c.hdt, 0, h.steps * 8, s));
    c.hsteps = h.steps;
    c.hper = h.per_step;
    c.hstride = h.stride;
  }
  DevState hs;
  std::memset(&hs, 0, sizeof(hs));
  hs.tf = a.tf;
  hs.cfl = a.cfl;
  hs.max_steps = a.max_steps > 0 ? a.max_steps : -1;
  hs.ndt = a.ndt;
  hs.snap_slot = -1;
  *ar->host_state = hs;
  CK(cudaMemcpyAsync(c.st, ar->host_state, sizeof(DevState),
                     cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c.u, a.u, usz * 8, cudaMemcpyHostToDevice, s));

  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  if (!a.profile) { // capture K steps into one graph
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaSuccess;
    for (int k = 0; k < K && ce == cudaSuccess; k++)
      ce = enqueue_step(c, s);
    cudaError_t ee = cudaStreamEndCapture(s, &graph);
    if (ce != cudaSuccess) {
      set_error(std::string("enqueue step: ") + cudaGetErrorString(ce));
      return PYPDE_ERR_CUDA;
    }
    CK(ee);
    CK(cudaGraphInstantiate(&exec, graph, 0));
  }
  cudaEvent_t pev[9];
  if (a.profile)
    for (int i = 0; i < 9; i++)
      CK(cudaEventCreate(&pev[i]));
  double stage_s[8] = {};
  long long launches = 0;

  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, s));
  int drained = 0;
  rc = PYPDE_OK;
  for (;;) {
    if (a.profile) {
      CK(enqueue_step(c, s, pev));
      launches += kernels_per_step(c, true);
    } else {
      CK(cudaGraphLaunch(exec, s));
      launches += (long long)K * kernels_per_step(c, false);
    }
    CK(cudaMemcpyAsync(ar->host_state, c.st, sizeof(DevState),
                       cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    DevState h = *ar->host_state;
    if (a.profile && h.active) {
      // stage i spans events (i, i+1); ghost fill .. gather are stages 0-6,
      // the bookkeeping kernels count as "other"
      for (int i = 0; i < 7; i++) {
        float ms = 0;
        cudaEventElapsedTime(&ms, pev[i], pev[i + 1]);
        stage_s[i] += ms * 1e-3;
      }
      float ms = 0;
      cudaEventElapsedTime(&ms, pev[7], pev[8]);
      stage_s[7] += ms * 1e-3;
    }
    // snapshots taken during this launch: ring slot p % ring holds row p
    for (; drained < h.push; drained++)
      if (a.ret)
        CK(cudaMemcpyAsync(a.ret + (long long)drained * usz,
                           c.ringbuf + (long long)(drained % c.ring) * usz,
                           usz * 8, cudaMemcpyDeviceToHost, s));
    bool more = (h.t < h.tf) && (h.max_steps < 0 || h.count < h.max_steps) &&
                !h.nan_found;
    if (h.nan_found) {
      if (a.ret && h.push < a.ndt)
        CK(cudaMemcpyAsync(a.ret + (long long)h.push * usz, c.uprev, usz * 8,
                           cudaMemcpyDeviceToHost, s));
      if (a.ret && h.push + 1 < a.ndt)
        CK(cudaMemcpyAsync(a.ret + (long long)(h.push + 1) * usz, c.u,
                           usz * 8, cudaMemcpyDeviceToHost, s));
      rc = PYPDE_NAN_FOUND;
    }
    if (!more)
      break;
  }
  CK(cudaEventRecord(e1, s));
  CK(cudaMemcpyAsync(a.u, c.u, usz * 8, cudaMemcpyDeviceToHost, s));
  if (c.hw) {
    long long rows = (long long)c.hsteps * c.hper;
    CK(cudaMemcpyAsync(a.harvest->w, c.hw, rows * Nd * V * 8,
                       cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(a.harvest->qh, c.hq, rows * N * Nd * V * 8,
                       cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(a.harvest->dt, c.hdt, c.hsteps * 8,
                       cudaMemcpyDeviceToHost, s));
  }
  if (a.ret)
    CK(cudaMemcpyAsync(a.ret + (long long)(a.ndt - 1) * usz, c.u, usz * 8,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (exec)
    cudaGraphExecDestroy(exec);
  if (graph)
    cudaGraphDestroy(graph);
  if (a.profile)
    for (int i = 0; i < 9; i++)
      cudaEventDestroy(pev[i]);
  DevState h = *ar->host_state;
  if (out) {
    out->steps = h.count;
    out->t_final = h.t;
    out->pred_iters = h.pred_iters;
    out->pred_max_iters = h.pred_max_iters;
    out->pred_fail = h.pred_fail;
    out->pred_fallbacks = h.pred_fallbacks;
    out->pred_iters32 = h.pred_iters32;
    out->nan_found = h.nan_found;
    out->device_seconds = ms * 1e-3;
    out->kernel_launches = launches;
    for (int i = 0; i < 8; i++)
      out->stage_seconds[i] = stage_s[i];
  }
  return rc;
}

// ------------------------------------------------------------------
// batched runs: many problems, one launch per stage and order (batch.cuh)
// ------------------------------------------------------------------
static const void *kb_weno_kernel(int N) {
  switch (N) {
  case 1: return (const void *)&kb_weno<1>;
  case 2: return (const void *)&kb_weno<2>;
  case 3: return (const void *)&kb_weno<3>;
  case 4: return (const void *)&kb_weno<4>;
  case 5: return (const void *)&kb_weno<5>;
  case 6: return (const void *)&kb_weno<6>;
  default: return nullptr;
  }
}

// CTAs of a kernel resident per SM (sizes the persistent grids).
static int resident_blocks(const KFunc &f, int threads, size_t smem) {
  int n = 0;
  if (f.aot) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f.aot, threads,
                                                      smem) != cudaSuccess)
      n = 1;
  } else if (f.jit) {
    typedef int (*occ_t)(int *, void *, int, size_t);
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(
            "cuOccupancyMaxActiveBlocksPerMultiprocessor", &p, 12000,
            cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || ((occ_t)p)(&n, f.jit, threads, smem))
      n = 1;
  }
  return n < 1 ? 1 : n;
}

namespace {
// Problems of one order, largest first.
struct BatchGroup {
  int N = 0;
  const KernelSet *ks = nullptr;
  Tables T;
  std::vector<int> idx;
  BatchProblem *dP = nullptr; // device, idx.size() entries
  long long *dOff[BS_COUNT] = {};
  long long tiles[BS_COUNT] = {};
  int per_pop[BS_COUNT] = {};
  KFunc fn[BS_COUNT];
  int threads[BS_COUNT] = {};
  size_t smem[BS_COUNT] = {};
  int resident[BS_COUNT] = {};
  // the faces stage in two launches (kb_faces_pre as fn[BS_FACES], then
  // this one over the same tiles, with its own queue)
  KFunc faces_eig;
  int faces_eig_resident = 0;
  bool guess = false; // a learned warm start for this order
  MlpModel model;
};

// Queue heads per group: one per stage, and one for the second launch of
// the two-launch faces.
constexpr int HEADS = BS_COUNT + 1;

struct BatchCtx {
  std::vector<BatchGroup> G;
  BatchProblem *dPall = nullptr;
  int np = 0, ndim = 1, nsm = 152;
  unsigned long long *heads = nullptr;
  bool stiff = false, faces = true, centers = true;
  int flux = 0, mixed = 0;
  double tol = 1e-12;
};
} // namespace

// One batched step.  With ev non-null, an event is recorded before and
// after every (group, stage) launch: ev[(g * BS_COUNT + stage) * 2 + 0/1].
static cudaError_t enqueue_batch_step(BatchCtx &c, cudaStream_t s,
                                      cudaEvent_t *ev = nullptr) {
  cudaError_t e = cudaMemsetAsync(
      c.heads, 0, sizeof(unsigned long long) * c.G.size() * HEADS, s);
  if (e != cudaSuccess)
    return e;
  const unsigned pb = (unsigned)((c.np + 127) / 128);
  kb_step_begin<<<pb, 128, 0, s>>>(c.dPall, c.np);
  auto stage = [&](size_t gi, int st, void *x0, void *x1,
                   void *x2) -> cudaError_t {
    BatchGroup &g = c.G[gi];
    if (g.tiles[st] == 0)
      return cudaSuccess;
    TileQueue q{g.dOff[st], (int)g.idx.size(), c.heads + gi * HEADS + st};
    int pp = g.per_pop[st] >= 0 ? g.per_pop[st] : 1;
    unsigned grid;
    if (pp == 0) { // one block per tile, no queue
      grid = (unsigned)g.tiles[st];
    } else {
      long long want = (g.tiles[st] + pp - 1) / pp;
      long long cap = (long long)g.resident[st] * c.nsm;
      grid = (unsigned)(want < cap ? want : cap);
    }
    void *args[8] = {(void *)&g.dP, (void *)&q, (void *)&pp, x0, x1, x2,
                     nullptr, nullptr};
    if (ev)
      cudaEventRecord(ev[(gi * BS_COUNT + st) * 2], s);
    cudaError_t r = launch(g.fn[st], dim3(grid), dim3(g.threads[st]),
                           g.smem[st], s, args);
    if (r == cudaSuccess && st == BS_FACES && g.faces_eig.valid()) {
      // the second launch of the faces: the same tiles, its own queue
      TileQueue q2{g.dOff[st], (int)g.idx.size(),
                   c.heads + gi * HEADS + BS_COUNT};
      unsigned grid2 = grid;
      if (pp != 0) {
        long long want = (g.tiles[st] + pp - 1) / pp;
        long long cap = (long long)g.faces_eig_resident * c.nsm;
        grid2 = (unsigned)(want < cap ? want : cap);
      }
      void *args2[3] = {(void *)&g.dP, (void *)&q2, (void *)&pp};
      r = launch(g.faces_eig, dim3(grid2), dim3(128), 0, s, args2);
    }
    if (ev)
      cudaEventRecord(ev[(gi * BS_COUNT + st) * 2 + 1], s);
    return r;
  };
  for (size_t gi = 0; gi < c.G.size(); gi++) {
    BatchGroup &g = c.G[gi];
    if ((e = stage(gi, BS_BOUNDARIES, nullptr, nullptr, nullptr)))
      return e;
    for (int d = 0; d < c.ndim; d++) {
      int dd = d;
      if ((e = stage(gi, BS_WENO0 + d, (void *)&dd, (void *)&g.T,
                     nullptr)))
        return e;
    }
    if ((e = stage(gi, BS_CFL, (void *)&g.T, nullptr, nullptr)))
      return e;
  }
  kb_dt<<<pb, 128, 0, s>>>(c.dPall, c.np);
  for (size_t gi = 0; gi < c.G.size(); gi++) {
    BatchGroup &g = c.G[gi];
    double tol = c.tol;
    int flags = (g.guess ? 1 : 0) | (c.mixed ? 2 : 0);
    if (g.guess &&
        (e = stage(gi, BS_GUESS, (void *)&g.model, nullptr, nullptr)))
      return e;
    if ((e = stage(gi, BS_PREDICTOR, (void *)&g.T,
                   c.stiff ? (void *)&tol : nullptr,
                   c.stiff ? (void *)&flags : nullptr)))
      return e;
    if (c.faces && (e = stage(gi, BS_FACES, (void *)&g.T, nullptr, nullptr)))
      return e;
    if (c.centers &&
        (e = stage(gi, BS_CENTERS, (void *)&g.T, nullptr, nullptr)))
      return e;
    int uc = c.centers ? 1 : 0, uf = c.faces ? 1 : 0;
    if ((e = stage(gi, BS_GATHER, (void *)&uc, (void *)&uf, nullptr)))
      return e;
  }
  kb_step_end<<<pb, 128, 0, s>>>(c.dPall, c.np);
  return cudaGetLastError();
}

static int batch_launches_per_step(const BatchCtx &c) {
  int n = 3;
  for (auto &g : c.G) {
    for (int st = 0; st < BS_COUNT; st++)
      if (g.tiles[st] > 0)
        n++;
    if (g.tiles[BS_FACES] > 0 && g.faces_eig.valid())
      n++; // the faces' second launch
  }
  return n;
}

int run_batch(const SystemDesc &sys, const BatchArgs &a, BatchStats *out) {
  NvtxRange nvtx_run("pde_solver_batch");
  if (a.np < 1 || !a.probs) {
    set_error("empty batch");
    return PYPDE_ERR_ARG;
  }
  const int ndim = sys.ndim, V = sys.V;
  for (int p = 0; p < a.np; p++) {
    const ProblemSpec &q = a.probs[p];
    if (!q.u || !(q.tf >= 0) || q.N < 1 || q.N > MAXN) {
      set_error("batch problem " + std::to_string(p) + ": invalid arguments");
      return PYPDE_ERR_ARG;
    }
    for (int d = 0; d < ndim; d++)
      if (q.nX[d] < 1 || !(q.dX[d] > 0) || (q.bt[d] != 0 && q.bt[d] != 1)) {
        set_error("batch problem " + std::to_string(p) + ": invalid grid");
        return PYPDE_ERR_ARG;
      }
    int rc = check_system(sys, ndim, q.N, a.stiff, a.flux);
    if (!rc)
      rc = check_grid(ndim, q.nX, q.bt, q.N);
    if (rc)
      return rc;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  Arena *ar;
  int rc = arena_for(a.device, &ar);
  if (rc)
    return rc;
  cudaStream_t s = ar->stream;
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, a.device));

  BatchCtx c;
  c.np = a.np;
  c.ndim = ndim;
  c.nsm = prop.multiProcessorCount;
  c.stiff = a.stiff;
  c.flux = a.flux;
  c.tol = a.newton_tol;
  c.mixed = a.mixed ? 1 : 0;
  c.faces = sys.has_F || sys.has_B;
  c.centers = sys.has_B || sys.has_S;

  // order groups, problems largest first within each
  std::vector<Geom> geo(a.np);
  std::vector<FaceIndex> fis(a.np);
  for (int p = 0; p < a.np; p++) {
    fill_geom(geo[p], ndim, a.probs[p].nX, a.probs[p].bt, a.probs[p].dX,
              a.probs[p].N);
    fis[p] = face_index(geo[p], a.probs[p].N);
  }
  for (int N = 1; N <= MAXN; N++) {
    BatchGroup g;
    for (int p = 0; p < a.np; p++)
      if (a.probs[p].N == N)
        g.idx.push_back(p);
    if (g.idx.empty())
      continue;
    if ((rc = ensure_kernels(sys, N)))
      return rc;
    g.N = N;
    g.ks = &sys.sets[N];
    if (!g.ks->kb_cfl.valid() || !kb_weno_kernel(N)) {
      set_error("no batched kernels for system " + sys.name + " at order " +
                std::to_string(N));
      return PYPDE_ERR_UNSUPPORTED;
    }
    make_tables(N, &g.T);
    if (a.warm[N]) {
      if ((rc = check_warm(sys, N, a.stiff, a.device, a.warm[N])))
        return rc;
      if (!g.ks->kb_guess.valid()) {
        set_error("no batched warm-start kernel for system " + sys.name);
        return PYPDE_ERR_UNSUPPORTED;
      }
      g.guess = true;
      g.model = a.warm[N]->model;
    }
    std::stable_sort(g.idx.begin(), g.idx.end(),
                     [&](int x, int y) { return geo[x].C > geo[y].C; });
    c.G.push_back(g);
  }

  // device memory: one region per buffer kind, carved per problem
  DeviceBuffers mem;
  std::vector<BatchProblem> hp(a.np);
  std::vector<size_t> o_u(a.np), o_ub(a.np), o_ta(a.np), o_tb(a.np),
      o_w(a.np), o_qh(a.np), o_ct(a.np), o_cen(a.np), o_wp(a.np);
  size_t t_u = 0, t_ub = 0, t_ta = 0, t_tb = 0, t_w = 0, t_qh = 0, t_ct = 0,
         t_cen = 0, t_wp = 0;
  auto carve = [](size_t &tot, size_t doubles) {
    size_t at = tot;
    tot += (doubles + 31) / 32 * 32; // 256-byte aligned
    return at;
  };
  // The Rusanov faces of a first-order flux system without B run in two
  // launches, through records of every face point of the batch (73 doubles
  // a point for the 2-D relaxation system: 76 GB for 256 problems of 64^2
  // to 512^2 cells and orders 1-3, within the GPU's memory).
  // Without room for them the faces run as one launch (recs_ok false).
  std::vector<size_t> o_rec(a.np);
  size_t t_rec = 0;
  bool recs_ok = true;
  auto two_launch_faces = [&](int N) {
    const KernelSet &k = sys.sets[N];
    return recs_ok && c.faces && a.flux == 0 && k.kb_faces_pre.valid() &&
           k.face_rec > 0;
  };
  for (int p = 0; p < a.np; p++) {
    const int N = a.probs[p].N, Nd = ipow(N, ndim);
    const Geom &g = geo[p];
    long long tmpn = weno_tmp_doubles(g.nXb, ndim, N, V);
    o_u[p] = carve(t_u, g.C * V);
    o_ub[p] = carve(t_ub, g.Cb * V);
    o_ta[p] = carve(t_ta, tmpn);
    o_tb[p] = carve(t_tb, tmpn);
    o_w[p] = carve(t_w, g.Cw * Nd * V);
    o_qh[p] = carve(t_qh, g.Cw * N * Nd * V);
    o_ct[p] = carve(t_ct, c.faces ? fis[p].off[ndim] * 2 * V : 1);
    o_cen[p] = carve(t_cen, c.centers ? g.C * N * Nd * V : 1);
    o_wp[p] = carve(t_wp, Nd);
    o_rec[p] = carve(t_rec, two_launch_faces(N)
                                ? fis[p].off[ndim] * sys.sets[N].face_rec
                                : 0);
  }
  double *b_u, *b_ub, *b_ta, *b_tb, *b_w, *b_qh, *b_ct, *b_cen, *b_wp;
  double *b_rec = nullptr;
  DevState *b_st;
  CK(mem.alloc((void **)&b_u, t_u * 8));
  CK(mem.alloc((void **)&b_ub, t_ub * 8));
  CK(mem.alloc((void **)&b_ta, t_ta * 8));
  CK(mem.alloc((void **)&b_tb, t_tb * 8));
  CK(mem.alloc((void **)&b_w, t_w * 8));
  CK(mem.alloc((void **)&b_qh, t_qh * 8));
  CK(mem.alloc((void **)&b_ct, t_ct * 8));
  CK(mem.alloc((void **)&b_cen, t_cen * 8));
  CK(mem.alloc((void **)&b_wp, t_wp * 8));
  if (t_rec == 0) {
    recs_ok = false;
  } else if (mem.alloc((void **)&b_rec, t_rec * 8) != cudaSuccess) {
    cudaGetLastError(); // the failed allocation
    recs_ok = false;
  }
  CK(mem.alloc((void **)&b_st, sizeof(DevState) * a.np));
  CK(mem.alloc((void **)&c.heads,
               sizeof(unsigned long long) * c.G.size() * HEADS));

  // problem descriptors and tile tables, in group order
  std::vector<BatchProblem> order;
  std::vector<DevState> hs(a.np);
  for (auto &g : c.G) {
    const int N = g.N, Nd = ipow(N, ndim), NT = N * Nd;
    const KernelSet &k = *g.ks;
    std::vector<long long> off[BS_COUNT];
    for (int st = 0; st < BS_COUNT; st++)
      off[st].push_back(0);
    for (int p : g.idx) {
      const Geom &ge = geo[p];
      BatchProblem b;
      b.g = ge;
      b.fi = fis[p];
      b.N = N;
      b.V = V;
      b.u = b_u + o_u[p];
      b.ub = b_ub + o_ub[p];
      b.w = b_w + o_w[p];
      b.qh = b_qh + o_qh[p];
      b.contrib = b_ct + o_ct[p];
      b.cen = b_cen + o_cen[p];
      b.wprod = b_wp + o_wp[p];
      b.rec = two_launch_faces(N) ? b_rec + o_rec[p] : nullptr;
      b.st = b_st + p;
      long long tw[3] = {0, 0, 0};
      int m[3] = {ge.nXb[0], ge.nXb[1], ge.nXb[2]};
      const double *src = b.ub;
      int n4 = 1;
      for (int d = 0; d < ndim; d++) {
        long long n1 = 1, n3 = 1;
        for (int e2 = 0; e2 < d; e2++)
          n1 *= m[e2];
        for (int e2 = d + 1; e2 < ndim; e2++)
          n3 *= m[e2];
        double *dst = (d == ndim - 1)
                          ? b.w
                          : ((d % 2 == 0) ? b_ta + o_ta[p] : b_tb + o_tb[p]);
        b.win[d] = src;
        b.wout[d] = dst;
        b.wn1[d] = n1;
        b.wn3[d] = n3;
        b.wmd[d] = m[d];
        b.wn4[d] = n4;
        tw[d] = n1 * (m[d] - 2 * (N - 1)) * n3 * (long long)n4 * V;
        src = dst;
        m[d] -= 2 * (N - 1);
        n4 *= N;
      }
      for (int d = ndim; d < 3; d++) {
        b.win[d] = nullptr;
        b.wout[d] = nullptr;
        b.wn1[d] = b.wn3[d] = 0;
        b.wmd[d] = b.wn4[d] = 0;
      }
      auto tiles = [](long long work, int per) { return (work + per - 1) / per; };
      long long tl[BS_COUNT] = {};
      tl[BS_BOUNDARIES] = tiles(ge.Cb * V, 256);
      for (int d = 0; d < ndim; d++)
        tl[BS_WENO0 + d] = tiles(tw[d], 128);
      tl[BS_CFL] = tiles(ge.Cw, 128);
      tl[BS_PREDICTOR] = tiles(ge.Cw, a.stiff ? k.newton_cpb : k.pred_cpb);
      tl[BS_FACES] = c.faces ? tiles(fis[p].off[ndim], 128) : 0;
      tl[BS_CENTERS] = c.centers ? tiles(ge.C * NT, 128) : 0;
      tl[BS_GATHER] = tiles(ge.C * V, 256);
      tl[BS_GUESS] = g.guess ? tiles(ge.Cw, 128) : 0; // MlpShape::CELLS
      for (int st = 0; st < BS_COUNT; st++)
        off[st].push_back(off[st].back() + tl[st]);
      order.push_back(b);
      DevState d0;
      std::memset(&d0, 0, sizeof(d0));
      d0.tf = a.probs[p].tf;
      d0.cfl = a.probs[p].cfl;
      d0.max_steps = a.max_steps > 0 ? a.max_steps : -1;
      d0.ndt = 1;
      d0.snap_slot = -1;
      hs[p] = d0;
    }
    for (int st = 0; st < BS_COUNT; st++) {
      g.tiles[st] = off[st].back();
      CK(mem.alloc((void **)&g.dOff[st], off[st].size() * 8));
      CK(cudaMemcpyAsync(g.dOff[st], off[st].data(), off[st].size() * 8,
                         cudaMemcpyHostToDevice, s));
      g.per_pop[st] = a.per_pop >= 0 ? a.per_pop : 1;
    }
    g.fn[BS_BOUNDARIES].aot = (const void *)&kb_boundaries;
    g.threads[BS_BOUNDARIES] = 256;
    for (int d = 0; d < 3; d++) {
      g.fn[BS_WENO0 + d].aot = kb_weno_kernel(N);
      g.threads[BS_WENO0 + d] = 128;
    }
    g.fn[BS_CFL] = k.kb_cfl;
    g.threads[BS_CFL] = 128;
    if (a.stiff) {
      g.fn[BS_PREDICTOR] = k.kb_newton;
      g.threads[BS_PREDICTOR] = k.newton_threads;
      g.smem[BS_PREDICTOR] = k.newton_smem;
    } else {
      g.fn[BS_PREDICTOR] = k.kb_predictor;
      g.threads[BS_PREDICTOR] = k.pred_threads;
      g.smem[BS_PREDICTOR] = k.pred_smem;
    }
    if (two_launch_faces(N)) {
      g.fn[BS_FACES] = k.kb_faces_pre;
      g.faces_eig = k.kb_faces_eig;
    } else {
      g.fn[BS_FACES] = k.kb_faces[a.flux];
    }
    g.threads[BS_FACES] = 128;
    g.fn[BS_CENTERS] = k.kb_centers;
    g.threads[BS_CENTERS] = 128;
    g.fn[BS_GATHER] = k.kb_gather;
    g.threads[BS_GATHER] = 256;
    if (g.guess) {
      g.fn[BS_GUESS] = k.kb_guess;
      g.threads[BS_GUESS] = 256;
      g.smem[BS_GUESS] = k.guess_smem;
    }
    for (int st = 0; st < BS_COUNT; st++) {
      if (g.tiles[st] == 0)
        continue;
      CK(set_smem(g.fn[st], g.smem[st]));
      g.resident[st] = resident_blocks(g.fn[st], g.threads[st], g.smem[st]);
    }
    if (g.faces_eig.valid())
      g.faces_eig_resident = resident_blocks(g.faces_eig, 128, 0);
  }
  CK(mem.alloc((void **)&c.dPall, sizeof(BatchProblem) * order.size()));
  CK(cudaMemcpyAsync(c.dPall, order.data(), sizeof(BatchProblem) * order.size(),
                     cudaMemcpyHostToDevice, s));
  {
    size_t at = 0;
    for (auto &g : c.G) {
      g.dP = c.dPall + at;
      at += g.idx.size();
    }
  }
  // the problems' DevStates sit at b_st + p: upload, then states and u
  CK(cudaMemcpyAsync(b_st, hs.data(), sizeof(DevState) * a.np,
                     cudaMemcpyHostToDevice, s));
  for (int p = 0; p < a.np; p++) {
    const int Nd = ipow(a.probs[p].N, ndim);
    std::vector<double> wp(Nd);
    Tables T;
    make_tables(a.probs[p].N, &T);
    make_wprod(T, ndim, wp.data());
    CK(cudaMemcpyAsync(b_wp + o_wp[p], wp.data(), Nd * 8,
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b_u + o_u[p], a.probs[p].u, geo[p].C * V * 8,
                       cudaMemcpyHostToDevice, s));
  }
  std::vector<DevState> host(a.np);
  auto all_done = [&]() -> cudaError_t {
    cudaError_t e2 = cudaMemcpyAsync(host.data(), b_st,
                                     sizeof(DevState) * a.np,
                                     cudaMemcpyDeviceToHost, s);
    if (e2 == cudaSuccess)
      e2 = cudaStreamSynchronize(s);
    return e2;
  };
  auto finished = [&]() {
    for (int p = 0; p < a.np; p++) {
      const DevState &h = host[p];
      if (h.t < h.tf && (h.max_steps < 0 || h.count < h.max_steps) &&
          !h.nan_found)
        return false;
    }
    return true;
  };

  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, s));
  long long launches = 0;
  double tune_s = 0;
  CK(all_done());
  // autotune: the first steps run eagerly, one tile shape per step (0: a
  // block per tile; 1-8: tiles per pop of the persistent queue), each
  // (group, stage) launch timed; the fastest shape per launch is kept
  if (a.autotune && !finished()) {
    const int cand[5] = {0, 1, 2, 4, 8};
    const size_t nev = c.G.size() * BS_COUNT * 2;
    std::vector<cudaEvent_t> ev(nev);
    for (auto &x : ev)
      CK(cudaEventCreate(&x));
    std::vector<float> best(c.G.size() * BS_COUNT, 1e30f);
    std::vector<int> pick(c.G.size() * BS_COUNT, 1);
    auto t0 = std::chrono::steady_clock::now();
    for (int ci = 0; ci < 5 && !finished(); ci++) {
      for (auto &g : c.G)
        for (int st = 0; st < BS_COUNT; st++)
          g.per_pop[st] = cand[ci];
      CK(enqueue_batch_step(c, s, ev.data()));
      launches += batch_launches_per_step(c);
      CK(all_done());
      for (size_t gi = 0; gi < c.G.size(); gi++)
        for (int st = 0; st < BS_COUNT; st++) {
          if (c.G[gi].tiles[st] == 0)
            continue;
          float ms = 0;
          if (cudaEventElapsedTime(&ms, ev[(gi * BS_COUNT + st) * 2],
                                   ev[(gi * BS_COUNT + st) * 2 + 1]) ==
                  cudaSuccess &&
              ms < best[gi * BS_COUNT + st]) {
            best[gi * BS_COUNT + st] = ms;
            pick[gi * BS_COUNT + st] = cand[ci];
          }
        }
    }
    for (size_t gi = 0; gi < c.G.size(); gi++)
      for (int st = 0; st < BS_COUNT; st++)
        c.G[gi].per_pop[st] = pick[gi * BS_COUNT + st];
    for (auto &x : ev)
      cudaEventDestroy(x);
    tune_s = std::chrono::duration<double>(std::chrono::steady_clock::now() -
                                           t0)
                 .count();
  }
  int K = a.steps_per_graph > 0 ? a.steps_per_graph : 8;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  if (!finished()) {
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaSuccess;
    for (int k = 0; k < K && ce == cudaSuccess; k++)
      ce = enqueue_batch_step(c, s);
    cudaError_t ee = cudaStreamEndCapture(s, &graph);
    if (ce != cudaSuccess) {
      if (graph)
        cudaGraphDestroy(graph);
      set_error(std::string("enqueue batched step: ") + cudaGetErrorString(ce));
      return PYPDE_ERR_CUDA;
    }
    CK(ee);
    CK(cudaGraphInstantiate(&exec, graph, 0));
    while (!finished()) {
      CK(cudaGraphLaunch(exec, s));
      launches += (long long)K * batch_launches_per_step(c);
      CK(all_done());
    }
  }
  CK(cudaEventRecord(e1, s));
  for (int p = 0; p < a.np; p++)
    CK(cudaMemcpyAsync(a.probs[p].u, b_u + o_u[p], geo[p].C * V * 8,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (exec)
    cudaGraphExecDestroy(exec);
  if (graph)
    cudaGraphDestroy(graph);
  if (out) {
    out->steps = 0;
    out->max_problem_steps = 0;
    out->pred_iters = 0;
    out->nan_found = 0;
    for (int p = 0; p < a.np; p++) {
      out->steps += host[p].count;
      out->max_problem_steps = std::max(out->max_problem_steps, host[p].count);
      out->pred_iters += host[p].pred_iters;
      out->nan_found += host[p].nan_found ? 1 : 0;
      if (out->steps_per_problem)
        out->steps_per_problem[p] = host[p].count;
      if (out->t_per_problem)
        out->t_per_problem[p] = host[p].t;
    }
    out->device_seconds = ms * 1e-3;
    out->kernel_launches = launches;
    out->tune_seconds = tune_s;
    for (int st = 0; st < BS_COUNT; st++)
      out->per_pop[st] = c.G.empty() ? 0 : c.G[0].per_pop[st];
  }
  int nan_any = 0;
  for (int p = 0; p < a.np; p++)
    nan_any |= host[p].nan_found;
  return nan_any ? PYPDE_NAN_FOUND : PYPDE_OK;
}

// ------------------------------------------------------------------
// single stages
// ------------------------------------------------------------------
static int put_state(Arena *ar, DevState **dst, double t, double tf,
                     double cfl, long long count, double dt) {
  CK(ensure(ar->state, sizeof(DevState)));
  DevState hs;
  std::memset(&hs, 0, sizeof(hs));
  hs.active = 1;
  hs.t = t;
  hs.tf = tf;
  hs.cfl = cfl;
  hs.count = count;
  hs.dt = dt;
  hs.max_steps = -1;
  hs.snap_slot = -1;
  *ar->host_state = hs;
  CK(cudaMemcpyAsync(ar->state.p, ar->host_state, sizeof(DevState),
                     cudaMemcpyHostToDevice, ar->stream));
  *dst = (DevState *)ar->state.p;
  return PYPDE_OK;
}

int stage_boundaries(const double *u, const int *nX, int ndim, const int *bt,
                     int N, int V, double *ub) {
  if (ndim < 1 || ndim > 3 || N < 1 || V < 1) {
    set_error("invalid arguments");
    return PYPDE_ERR_ARG;
  }
  int rc = check_grid(ndim, nX, bt, N);
  if (rc)
    return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  Arena *ar;
  rc = arena_for(0, &ar);
  if (rc)
    return rc;
  Geom g;
  fill_geom(g, ndim, nX, bt, nullptr, N);
  DevState *st;
  if ((rc = put_state(ar, &st, 0, 1, 1, 0, 0)))
    return rc;
  CK(ensure(ar->u, g.C * V * 8));
  CK(ensure(ar->ub, g.Cb * V * 8));
  cudaStream_t s = ar->stream;
  CK(cudaMemcpyAsync(ar->u.p, u, g.C * V * 8, cudaMemcpyHostToDevice, s));
  k_boundaries<<<grid_for(g.Cb * V, 256, 152 * 32), 256, 0, s>>>(
      (double *)ar->u.p, (double *)ar->ub.p, g, N, V, st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ub, ar->ub.p, g.Cb * V * 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return PYPDE_OK;
}

int stage_weno(const double *ubh, const int *nXb, int ndim, int N, int V,
               double *wh) {
  if (ndim < 1 || ndim > 3 || N < 1 || N > 6 || V < 1) {
    set_error("invalid arguments (WENO is built for N <= 6)");
    return PYPDE_ERR_ARG;
  }
  long long cin = 1, cout = 1;
  for (int d = 0; d < ndim; d++) {
    if (nXb[d] - 2 * (N - 1) < 1) {
      set_error("grid too small for this order");
      return PYPDE_ERR_ARG;
    }
    cin *= nXb[d];
    cout *= nXb[d] - 2 * (N - 1);
  }
  std::lock_guard<std::mutex> lock(g_mu);
  Arena *ar;
  int rc = arena_for(0, &ar);
  if (rc)
    return rc;
  DevState *st;
  if ((rc = put_state(ar, &st, 0, 1, 1, 0, 0)))
    return rc;
  long long nout = cout * ipow(N, ndim) * V;
  long long tmpn = weno_tmp_doubles(nXb, ndim, N, V);
  CK(ensure(ar->ub, cin * V * 8));
  CK(ensure(ar->w, nout * 8));
  CK(ensure(ar->tmpA, tmpn * 8));
  CK(ensure(ar->tmpB, tmpn * 8));
  Tables T;
  make_tables(N, &T);
  cudaStream_t s = ar->stream;
  CK(cudaMemcpyAsync(ar->ub.p, ubh, cin * V * 8, cudaMemcpyHostToDevice, s));
  CK(enqueue_weno((double *)ar->ub.p, nXb, ndim, N, V, T,
                  (double *)ar->tmpA.p, (double *)ar->tmpB.p,
                  (double *)ar->w.p, st, s));
  CK(cudaMemcpyAsync(wh, ar->w.p, nout * 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return PYPDE_OK;
}

int stage_timestep(const SystemDesc &sys, const double *w, long long nrows,
                   const double *dX, int ndim, int N, double cfl, double tf,
                   double t, long long count, double *dt) {
  int rc = check_system(sys, ndim, N, false, 0);
  if (rc)
    return rc;
  int Nd = ipow(N, ndim);
  if (nrows < 1 || nrows % Nd) {
    set_error("nrows must be a positive multiple of N^ndim");
    return PYPDE_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  Arena *ar;
  if ((rc = arena_for(0, &ar)))
    return rc;
  if ((rc = ensure_kernels(sys, N)))
    return rc;
  DevState *st;
  if ((rc = put_state(ar, &st, t, tf, cfl, count, 0)))
    return rc;
  Geom g;
  int ones[3] = {1, 1, 1};
  fill_geom(g, ndim, ones, nullptr, dX, N);
  g.Cw = nrows / Nd;
  Tables T;
  make_tables(N, &T);
  std::vector<double> wp(Nd);
  make_wprod(T, ndim, wp.data());
  CK(ensure(ar->w, nrows * sys.V * 8));
  CK(ensure(ar->wprod, Nd * 8));
  cudaStream_t s = ar->stream;
  CK(cudaMemcpyAsync(ar->w.p, w, nrows * sys.V * 8, cudaMemcpyHostToDevice,
                     s));
  CK(cudaMemcpyAsync(ar->wprod.p, wp.data(), Nd * 8, cudaMemcpyHostToDevice,
                     s));
  double *wd = (double *)ar->w.p, *wpd = (double *)ar->wprod.p;
  void *a[] = {(void *)&wd, (void *)&g, (void *)&T, (void *)&wpd,
               (void *)&st};
  CK(launch(sys.sets[N].cfl, dim3(grid_for(g.Cw, 128, 152 * 64)), dim3(128),
            0, s, a));
  k_dt<<<1, 1, 0, s>>>(st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ar->host_state, st, sizeof(DevState),
                     cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *dt = ar->host_state->dt;
  return PYPDE_OK;
}

int stage_predictor(const SystemDesc &sys, const double *w, long long nrows,
                    const double *dX, int ndim, int N, bool stiff, double dt,
                    double tol, double *qh, Stats *out, const double *guess,
                    const WarmStart *warm) {
  int rc = check_system(sys, ndim, N, stiff, 0);
  if (rc)
    return rc;
  if ((guess || warm) && !stiff) {
    set_error("an initial guess applies to the stiff predictor only");
    return PYPDE_ERR_ARG;
  }
  int Nd = ipow(N, ndim);
  if (nrows < 1 || nrows % Nd) {
    set_error("nrows must be a positive multiple of N^ndim");
    return PYPDE_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  Arena *ar;
  if ((rc = arena_for(0, &ar)))
    return rc;
  if ((rc = ensure_kernels(sys, N)))
    return rc;
  if (warm && (rc = check_warm(sys, N, stiff, 0, warm)))
    return rc;
  DevState *st;
  if ((rc = put_state(ar, &st, 0, 1, 1, 0, dt)))
    return rc;
  StepCtx c;
  std::memset(&c, 0, sizeof(c));
  c.sys = &sys;
  c.ks = &sys.sets[N];
  int ones[3] = {1, 1, 1};
  fill_geom(c.g, ndim, ones, nullptr, dX, N);
  c.g.Cw = nrows / Nd;
  make_tables(N, &c.T);
  c.N = N;
  c.V = sys.V;
  c.stiff = stiff;
  c.tol = tol;
  std::vector<double> wp(Nd);
  make_wprod(c.T, ndim, wp.data());
  CK(ensure(ar->w, nrows * sys.V * 8));
  CK(ensure(ar->qh, nrows * N * sys.V * 8));
  CK(ensure(ar->wprod, Nd * 8));
  cudaStream_t s = ar->stream;
  CK(cudaMemcpyAsync(ar->w.p, w, nrows * sys.V * 8, cudaMemcpyHostToDevice,
                     s));
  CK(cudaMemcpyAsync(ar->wprod.p, wp.data(), Nd * 8, cudaMemcpyHostToDevice,
                     s));
  c.w = (double *)ar->w.p;
  c.qh = (double *)ar->qh.p;
  c.wprod = (double *)ar->wprod.p;
  c.st = st;
  c.warm = warm;
  c.guess = guess;
  if (guess)
    CK(cudaMemcpyAsync(c.qh, guess, nrows * N * sys.V * 8,
                       cudaMemcpyHostToDevice, s));
  if (warm)
    CK(set_smem(c.ks->guess, c.ks->guess_smem));
  CK(set_smem(stiff ? c.ks->newton : c.ks->predictor,
              stiff ? c.ks->newton_smem : c.ks->pred_smem));
  CK(enqueue_predictor(c, s));
  CK(cudaMemcpyAsync(qh, c.qh, nrows * N * sys.V * 8, cudaMemcpyDeviceToHost,
                     s));
  CK(cudaMemcpyAsync(ar->host_state, st, sizeof(DevState),
                     cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (out) {
    out->pred_iters = ar->host_state->pred_iters;
    out->pred_max_iters = ar->host_state->pred_max_iters;
    out->pred_fail = ar->host_state->pred_fail;
    out->pred_fallbacks = ar->host_state->pred_fallbacks;
  }
  return PYPDE_OK;
}

int stage_fv(const SystemDesc &sys, double *u, const double *qh,
             const int *nX, const double *dX, int ndim, int N, int flux,
             double dt) {
  int rc = check_system(sys, ndim, N, false, flux);
  if (rc)
    return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  Arena *ar;
  if ((rc = arena_for(0, &ar)))
    return rc;
  if ((rc = ensure_kernels(sys, N)))
    return rc;
  DevState *st;
  if ((rc = put_state(ar, &st, 0, 1, 1, 0, dt)))
    return rc;
  StepCtx c;
  std::memset(&c, 0, sizeof(c));
  c.sys = &sys;
  c.ks = &sys.sets[N];
  fill_geom(c.g, ndim, nX, nullptr, dX, N);
  c.fi = face_index(c.g, N);
  make_tables(N, &c.T);
  c.N = N;
  c.V = sys.V;
  c.faces = sys.has_F || sys.has_B;
  c.centers = sys.has_B || sys.has_S;
  c.flux = flux;
  int Nd = ipow(N, ndim);
  long long usz = c.g.C * c.V, qsz = c.g.Cw * N * Nd * c.V;
  CK(ensure(ar->u, usz * 8));
  CK(ensure(ar->qh, qsz * 8));
  CK(ensure(ar->contrib, (c.faces ? c.fi.off[ndim] : 1) * 2 * c.V * 8));
  CK(ensure(ar->cen, (c.centers ? c.g.C * N * Nd : 1) * c.V * 8));
  cudaStream_t s = ar->stream;
  CK(cudaMemcpyAsync(ar->u.p, u, usz * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ar->qh.p, qh, qsz * 8, cudaMemcpyHostToDevice, s));
  c.u = (double *)ar->u.p;
  c.qh = (double *)ar->qh.p;
  c.contrib = (double *)ar->contrib.p;
  c.cen = (double *)ar->cen.p;
  c.st = st;
  CK(enqueue_fv(c, s));
  CK(cudaMemcpyAsync(u, ar->u.p, usz * 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return PYPDE_OK;
}

// ------------------------------------------------------------------
// FP64 throughput of this GPU: the roofline denominator of the FP64-bound
// kernels (independent FMA chains, 8 per thread, 8 blocks per SM).
// ------------------------------------------------------------------
__global__ void k_dfma_peak(double *out, double a, double b, int iters) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b);
    x3 = fma(x3, a, b); x4 = fma(x4, a, b); x5 = fma(x5, a, b);
    x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] =
      x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

int measure_fp64(int device, double *tflops) {
  std::lock_guard<std::mutex> lock(g_mu);
  Arena *ar;
  int rc = arena_for(device, &ar);
  if (rc)
    return rc;
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int blocks = sms * 8, threads = 256, iters = 4096;
  Buf out;
  CK(ensure(out, (size_t)blocks * threads * 8));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    CK(cudaEventRecord(e0, ar->stream));
    k_dfma_peak<<<blocks, threads, 0, ar->stream>>>((double *)out.p, 0.999,
                                                     1e-3, iters);
    CK(cudaEventRecord(e1, ar->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best)
      best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out.p);
  *tflops = 2.0 * 8 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return PYPDE_OK;
}

// FP64 tensor-core throughput: every warp runs 4 independent chains of
// mma.sync m8n8k4 (D = A B + C, FP64), 8 x 8 x 4 FMAs each.  The study of
// moving the predictor's contractions to DMMA asks whether this rate is
// above the FMA pipe's at all.
__global__ void k_dmma_peak(double *out, double a0, int iters) {
  double a = a0 + (threadIdx.x & 7) * 1e-6, b = 1.0 - (threadIdx.x & 3) * 1e-7;
  double c[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 4; k++)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 "
                   "{%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] =
      c[0][0] + c[0][1] + c[1][0] + c[1][1] + c[2][0] + c[2][1] + c[3][0] +
      c[3][1];
}

int measure_dmma(int device, double *tflops) {
  std::lock_guard<std::mutex> lock(g_mu);
  Arena *ar;
  int rc = arena_for(device, &ar);
  if (rc)
    return rc;
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int blocks = sms * 8, threads = 256, iters = 1024;
  Buf out;
  CK(ensure(out, (size_t)blocks * threads * 8));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    CK(cudaEventRecord(e0, ar->stream));
    k_dmma_peak<<<blocks, threads, 0, ar->stream>>>((double *)out.p, 1e-3,
                                                     iters);
    CK(cudaEventRecord(e1, ar->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best)
      best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out.p);
  const double warps = (double)blocks * threads / 32;
  *tflops = 2.0 * 8 * 8 * 4 * 4 * iters * warps / (best * 1e-3) / 1e12;
  return PYPDE_OK;
}

} // namespace pypde
