// noalloc.cu -- WENO reconstruction on caller-owned device buffers, with no
// device allocation of its own.
//
// Who needs this: host code that runs inside another framework's device
// memory budget (a caching allocator that owns all of the GPU's memory, so a
// raw cudaMalloc either fails or breaks its accounting), and code on
// latency-critical paths where cudaMalloc/cudaFree are not allowed because
// they synchronise the device.  Such callers allocate their inputs and
// outputs themselves and cannot give the library a workspace.  The WENO
// reconstruction of a 2-D or 3-D grid needs scratch memory between its
// per-axis passes; here that scratch is a file-scope __device__ array of a
// fixed size, which every GPU that loads the library holds until the process
// exits.
#include "../../include/pypde_gb300.h"
#include "runtime.h"

#include <mutex>
#include <string>

namespace pypde {

// Maximum scratch: 4 Mi doubles (32 MiB) for the intermediate WENO passes.
constexpr long long NOALLOC_SCRATCH_DOUBLES = 4LL << 20;

static __device__ __align__(256) double g_weno_scratch[NOALLOC_SCRATCH_DOUBLES];

// k_weno_pass reads the step flag of a DevState; this one is permanently
// active (fields in declaration order: t, dt, tf, cfl, max_speed, count,
// max_steps, active).
static __device__ DevState g_noalloc_state = {0.0, 0.0, 0.0, 0.0, 0.0, 0, 0, 1};

constexpr int NOALLOC_MAX_DEVICES = 64;
static double *g_scratch_ptr[NOALLOC_MAX_DEVICES];
static DevState *g_state_ptr[NOALLOC_MAX_DEVICES];
static int g_sm_count[NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mu;

// Device addresses of the two symbols on the current device and its SM
// count, looked up once per device.
static int noalloc_setup(double **scratch, DevState **state, int *sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return PYPDE_ERR_CUDA;
  }
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
    set_error("weno_solver_noalloc: device ordinal out of range");
    return PYPDE_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_weno_scratch);
    if (e != cudaSuccess) {
      set_error(std::string("cudaGetSymbolAddress(scratch): ") +
                cudaGetErrorString(e));
      return PYPDE_ERR_CUDA;
    }
    void *q = nullptr;
    e = cudaGetSymbolAddress(&q, g_noalloc_state);
    if (e != cudaSuccess) {
      set_error(std::string("cudaGetSymbolAddress(state): ") +
                cudaGetErrorString(e));
      return PYPDE_ERR_CUDA;
    }
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || n < 1) {
      set_error(std::string("cudaDeviceGetAttribute(SM count): ") +
                cudaGetErrorString(e));
      return PYPDE_ERR_CUDA;
    }
    g_sm_count[dev] = n;
    g_scratch_ptr[dev] = (double *)p;
    g_state_ptr[dev] = (DevState *)q;
  }
  *scratch = g_scratch_ptr[dev];
  *state = g_state_ptr[dev];
  *sms = g_sm_count[dev];
  return PYPDE_OK;
}

static const void *weno_pass_kernel(int N) {
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

static int weno_noalloc(double *w, const double *ub, const int *nXb, int ndim,
                        int N, int V, cudaStream_t stream) {
  if (!w || !ub || !nXb || ndim < 1 || ndim > 3 || N < 1 || N > 6 ||
      V < 1) {
    set_error("weno_solver_noalloc: invalid arguments (ndim 1-3, N 1-6)");
    return PYPDE_ERR_ARG;
  }
  // shapes of the intermediate passes (all but the last go to scratch)
  long long m[3], off[2] = {0, 0}, need = 0;
  for (int d = 0; d < ndim; d++) {
    m[d] = nXb[d];
    if (m[d] - 2 * (N - 1) < 1) {
      set_error("weno_solver_noalloc: grid too small for this order");
      return PYPDE_ERR_ARG;
    }
  }
  {
    long long mm[3] = {m[0], m[1], m[2]}, n4 = 1;
    for (int d = 0; d < ndim - 1; d++) {
      mm[d] -= 2 * (N - 1);
      n4 *= N;
      long long sz = n4 * V;
      for (int e = 0; e < ndim; e++)
        sz *= mm[e];
      off[d] = need;
      need += (sz + 31) / 32 * 32; // keep each pass 256-byte aligned
    }
  }
  if (need > NOALLOC_SCRATCH_DOUBLES) {
    set_error("weno_solver_noalloc: the intermediate passes need " +
              std::to_string(need) + " doubles of scratch; the limit is " +
              std::to_string(NOALLOC_SCRATCH_DOUBLES) +
              " (32 MiB). Use weno_solver for larger grids.");
    return PYPDE_ERR_ARG;
  }
  double *scratch;
  DevState *st;
  int sms;
  int rc = noalloc_setup(&scratch, &st, &sms);
  if (rc)
    return rc;
  Tables T;
  make_tables(N, &T);
  const void *fn = weno_pass_kernel(N);
  const double *src = ub;
  int n4 = 1;
  for (int d = 0; d < ndim; d++) {
    long long n1 = 1, n3 = 1;
    for (int e = 0; e < d; e++)
      n1 *= m[e];
    for (int e = d + 1; e < ndim; e++)
      n3 *= m[e];
    int md = (int)m[d];
    double *dst = (d == ndim - 1) ? w : scratch + off[d];
    long long total = n1 * (md - 2 * (N - 1)) * n3 * (long long)n4 * V;
    long long blocks = (total + 127) / 128;
    if (blocks > (long long)sms * 64) // a grid-stride loop: 64 blocks per SM
      blocks = (long long)sms * 64;
    if (blocks < 1)
      blocks = 1;
    void *args[] = {(void *)&src, (void *)&dst, (void *)&n1, (void *)&md,
                    (void *)&n3,  (void *)&n4,  (void *)&V,  (void *)&T,
                    (void *)&st};
    cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)blocks), dim3(128),
                                     args, 0, stream);
    if (e != cudaSuccess) {
      set_error(std::string("weno_solver_noalloc launch: ") +
                cudaGetErrorString(e));
      return PYPDE_ERR_CUDA;
    }
    src = dst;
    m[d] -= 2 * (N - 1);
    n4 *= N;
  }
  return PYPDE_OK;
}

} // namespace pypde

extern "C" int weno_solver_noalloc(double *ret_dev, const double *u_dev,
                                   const int *nX, int ndim, int N, int V,
                                   void *stream) {
  return pypde::weno_noalloc(ret_dev, u_dev, nX, ndim, N, V,
                             (cudaStream_t)stream);
}
