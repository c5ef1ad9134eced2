// jit.cpp -- run-time compilation of user callback systems.
//
// The reference compiles the user's Python callbacks into host cfuncs with
// numba (pypde/cfuncs.py:30-75).  Here pypde_gb300/translate.py turns them
// into a CUDA C++ `struct UserSystem`, and this file compiles the same kernel
// templates as the built-in systems (kernels.cuh) for it with NVRTC, at the
// order N a run asks for, and loads the cubin through the driver API.
// libnvrtc is opened with dlopen on first use, so the library itself loads
// (and serves the built-in systems) without it.  Cubins are cached on disk
// under $PYPDE_GB300_CACHE (default ~/.cache/pypde_gb300), keyed by a hash of
// the program text, the options and the NVRTC version.
#include "../../include/pypde_gb300.h"
#include "runtime.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <dlfcn.h>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

namespace pypde {

namespace {

// ---- NVRTC, loaded at run time -------------------------------------------
typedef struct _nvrtcProgram *nvrtcProgram;
struct Nvrtc {
  void *h = nullptr;
  int (*create)(nvrtcProgram *, const char *, const char *, int,
                const char *const *, const char *const *);
  int (*compile)(nvrtcProgram, int, const char *const *);
  int (*log_size)(nvrtcProgram, size_t *);
  int (*log)(nvrtcProgram, char *);
  int (*cubin_size)(nvrtcProgram, size_t *);
  int (*cubin)(nvrtcProgram, char *);
  int (*add_name)(nvrtcProgram, const char *);
  int (*lowered)(nvrtcProgram, const char *, const char **);
  int (*destroy)(nvrtcProgram *);
  int (*version)(int *, int *);
};

Nvrtc *nvrtc() {
  static Nvrtc n;
  static bool tried = false;
  if (tried)
    return n.h ? &n : nullptr;
  tried = true;
  const char *names[] = {"libnvrtc.so.13", "libnvrtc.so",
                         "/usr/local/cuda/lib64/libnvrtc.so.13",
                         "/usr/local/cuda/lib64/libnvrtc.so"};
  for (const char *nm : names)
    if ((n.h = dlopen(nm, RTLD_NOW | RTLD_LOCAL)))
      break;
  if (!n.h)
    return nullptr;
#define SYM(f, s)                                                              \
  if (!(*(void **)&n.f = dlsym(n.h, s))) {                                     \
    n.h = nullptr;                                                             \
    return nullptr;                                                            \
  }
  SYM(create, "nvrtcCreateProgram");
  SYM(compile, "nvrtcCompileProgram");
  SYM(log_size, "nvrtcGetProgramLogSize");
  SYM(log, "nvrtcGetProgramLog");
  SYM(cubin_size, "nvrtcGetCUBINSize");
  SYM(cubin, "nvrtcGetCUBIN");
  SYM(add_name, "nvrtcAddNameExpression");
  SYM(lowered, "nvrtcGetLoweredName");
  SYM(destroy, "nvrtcDestroyProgram");
  SYM(version, "nvrtcVersion");
#undef SYM
  return &n;
}

// ---- driver API entry points ----------------------------------------------
void *drv(const char *name) {
  void *p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault,
                                       &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return p;
}

// ---- files -----------------------------------------------------------------
std::string lib_dir() {
  Dl_info info;
  if (dladdr((void *)&lib_dir, &info) && info.dli_fname) {
    std::string p = info.dli_fname;
    size_t k = p.rfind('/');
    return k == std::string::npos ? std::string(".") : p.substr(0, k);
  }
  return ".";
}

bool read_file(const std::string &path, std::string *out) {
  std::ifstream f(path, std::ios::binary);
  if (!f)
    return false;
  std::stringstream ss;
  ss << f.rdbuf();
  *out = ss.str();
  return true;
}

std::string cache_dir() {
  const char *e = getenv("PYPDE_GB300_CACHE");
  std::string d;
  if (e && *e)
    d = e;
  else {
    const char *home = getenv("HOME");
    d = std::string(home ? home : "/tmp") + "/.cache/pypde_gb300";
  }
  std::string cur;
  for (size_t i = 0; i < d.size(); i++) { // mkdir -p
    cur += d[i];
    if (d[i] == '/' || i + 1 == d.size())
      mkdir(cur.c_str(), 0755);
  }
  return d;
}

unsigned long long fnv1a(const std::string &s) {
  unsigned long long h = 1469598103934665603ULL;
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ULL;
  }
  return h;
}

struct JitInfo {
  std::string src;
  void *modules[MAXN + 1] = {};
};

std::mutex g_jit_mu;

const char *KERNELS[] = {"k_cfl",       "k_predictor", "k_newton",
                         "k_faces0",    "k_faces1",    "k_faces2",
                         "k_centers",   "k_gather",    "k_mlp_guess",
                         "kb_cfl",      "kb_predictor", "kb_newton",
                         "kb_faces0",   "kb_faces1",   "kb_faces2",
                         "kb_centers",  "kb_gather",   "kb_mlp_guess"};

} // namespace

// Compile (or load from the cache) the kernels of a run-time system at
// order N and fill d->sets[N].
int jit_ensure(SystemDesc &d, int N) {
  std::lock_guard<std::mutex> lock(g_jit_mu);
  if (d.have[N])
    return PYPDE_OK;
  JitInfo *ji = (JitInfo *)d.module;
  if (!ji) {
    set_error("system has no run-time source");
    return PYPDE_ERR_ARG;
  }
  std::string dir = lib_dir() + "/csrc/";
  const char *hdrs[] = {"kernels.cuh", "ader_common.cuh", "eig_full.cuh",
                        "mlp.cuh", "batch.cuh"};
  const int nh = 5;
  std::vector<std::string> hsrc(nh);
  for (int i = 0; i < nh; i++)
    if (!read_file(dir + hdrs[i], &hsrc[i])) {
      set_error("cannot read " + dir + hdrs[i]);
      return PYPDE_ERR_COMPILE;
    }
  std::string ns = std::to_string(N);
  std::string sh = "pypde::MlpShape<UserSystem, " + ns + ">";
  std::string prog = "#include \"mlp.cuh\"\n#include \"batch.cuh\"\n" + ji->src +
                     "\n__constant__ int pypde_cfg[11] = {"
                     "pypde::PredCfg<UserSystem, " + ns + ">::THREADS, "
                     "pypde::PredCfg<UserSystem, " + ns + ">::CPB, "
                     "pypde::PredCfg<UserSystem, " + ns + ">::SMEM_DOUBLES * 8, "
                     "pypde::NewtonCfg<UserSystem, " + ns + ">::THREADS, "
                     "pypde::NewtonCfg<UserSystem, " + ns + ">::CPB, "
                     "(int)pypde::NewtonCfg<UserSystem, " + ns +
                     ">::SMEM_BYTES, "
                     "(" + sh + "::OK && UserSystem::HAS_S) ? 1 : 0, "
                     "(int)" + sh + "::SMEM, " + sh + "::K1, " + sh + "::NO, " +
                     sh + "::FEAT};\n";
  std::vector<std::string> exprs = {
      "&pypde::k_cfl<UserSystem, " + ns + ">",
      "&pypde::k_predictor<UserSystem, " + ns + ">",
      "&pypde::k_newton<UserSystem, " + ns + ">",
      "&pypde::k_faces<UserSystem, " + ns + ", 0>",
      "&pypde::k_faces<UserSystem, " + ns + ", 1>",
      "&pypde::k_faces<UserSystem, " + ns + ", 2>",
      "&pypde::k_centers<UserSystem, " + ns + ">",
      "&pypde::k_gather<UserSystem, " + ns + ">",
      "&pypde::k_mlp_guess<UserSystem, " + ns + ">",
      "&pypde::kb_cfl<UserSystem, " + ns + ">",
      "&pypde::kb_predictor<UserSystem, " + ns + ">",
      "&pypde::kb_newton<UserSystem, " + ns + ">",
      "&pypde::kb_faces<UserSystem, " + ns + ", 0>",
      "&pypde::kb_faces<UserSystem, " + ns + ", 1>",
      "&pypde::kb_faces<UserSystem, " + ns + ", 2>",
      "&pypde::kb_centers<UserSystem, " + ns + ">",
      "&pypde::kb_gather<UserSystem, " + ns + ">",
      "&pypde::kb_mlp_guess<UserSystem, " + ns + ">"};
  const char *opts[] = {"--gpu-architecture=sm_103a", "-std=c++17",
                        "--fmad=false", "-lineinfo", "-DPYPDE_JIT=1"};
  const int nopts = 5;

  Nvrtc *nv = nvrtc();
  if (!nv) {
    set_error("libnvrtc could not be loaded: run-time compiled callbacks "
              "need the CUDA toolkit's NVRTC");
    return PYPDE_ERR_COMPILE;
  }
  int vmaj = 0, vmin = 0;
  nv->version(&vmaj, &vmin);
  std::string keytext = prog;
  for (auto &h : hsrc)
    keytext += h;
  for (int i = 0; i < nopts; i++)
    keytext += opts[i];
  keytext += std::to_string(vmaj) + "." + std::to_string(vmin);
  char key[32];
  snprintf(key, sizeof(key), "%016llx", fnv1a(keytext));
  std::string cpath = cache_dir() + "/" + key + ".cubin";
  std::string lpath = cache_dir() + "/" + key + ".names";

  std::string cubin, names;
  std::vector<std::string> lowered(exprs.size());
  if (read_file(cpath, &cubin) && read_file(lpath, &names)) {
    std::istringstream is(names);
    for (auto &l : lowered)
      std::getline(is, l);
  } else {
    nvrtcProgram p;
    const char *hp[nh] = {hsrc[0].c_str(), hsrc[1].c_str(), hsrc[2].c_str(),
                          hsrc[3].c_str(), hsrc[4].c_str()};
    if (nv->create(&p, prog.c_str(), "user_system.cu", nh, hp, hdrs) != 0) {
      set_error("nvrtcCreateProgram failed");
      return PYPDE_ERR_COMPILE;
    }
    for (auto &e : exprs)
      nv->add_name(p, e.c_str());
    int rc = nv->compile(p, nopts, opts);
    size_t ls = 0;
    nv->log_size(p, &ls);
    std::string log(ls, '\0');
    if (ls)
      nv->log(p, &log[0]);
    if (rc != 0) {
      nv->destroy(&p);
      set_error("NVRTC compilation of the callbacks failed:\n" + log);
      return PYPDE_ERR_COMPILE;
    }
    size_t cs = 0;
    nv->cubin_size(p, &cs);
    cubin.resize(cs);
    nv->cubin(p, &cubin[0]);
    names.clear();
    for (size_t i = 0; i < exprs.size(); i++) {
      const char *ln = nullptr;
      nv->lowered(p, exprs[i].c_str(), &ln);
      lowered[i] = ln ? ln : "";
      names += lowered[i] + "\n";
    }
    nv->destroy(&p);
    std::ofstream(cpath, std::ios::binary) << cubin;
    std::ofstream(lpath) << names;
  }

  // load the module into the current device's primary context
  typedef int (*load_t)(void **, const void *);
  typedef int (*getfn_t)(void **, void *, const char *);
  typedef int (*getglob_t)(unsigned long long *, size_t *, void *,
                           const char *);
  load_t load = (load_t)drv("cuModuleLoadData");
  getfn_t getfn = (getfn_t)drv("cuModuleGetFunction");
  getglob_t getglob = (getglob_t)drv("cuModuleGetGlobal");
  if (!load || !getfn || !getglob) {
    set_error("CUDA driver entry points unavailable");
    return PYPDE_ERR_CUDA;
  }
  cudaError_t ce = cudaFree(0); // make the primary context current
  if (ce != cudaSuccess) {
    set_error(std::string("CUDA: ") + cudaGetErrorString(ce));
    return PYPDE_ERR_CUDA;
  }
  void *mod = nullptr;
  if (load(&mod, cubin.data()) != 0) {
    set_error("cuModuleLoadData failed for the compiled callbacks");
    return PYPDE_ERR_CUDA;
  }
  ji->modules[N] = mod;
  KFunc *slots[] = {&d.sets[N].cfl,           &d.sets[N].predictor,
                    &d.sets[N].newton,        &d.sets[N].faces_flux[0],
                    &d.sets[N].faces_flux[1], &d.sets[N].faces_flux[2],
                    &d.sets[N].centers,       &d.sets[N].gather,
                    &d.sets[N].guess,         &d.sets[N].kb_cfl,
                    &d.sets[N].kb_predictor,  &d.sets[N].kb_newton,
                    &d.sets[N].kb_faces[0],   &d.sets[N].kb_faces[1],
                    &d.sets[N].kb_faces[2],   &d.sets[N].kb_centers,
                    &d.sets[N].kb_gather,     &d.sets[N].kb_guess};
  for (size_t i = 0; i < exprs.size(); i++) {
    void *f = nullptr;
    if (lowered[i].empty() || getfn(&f, mod, lowered[i].c_str()) != 0) {
      set_error(std::string("kernel missing from compiled module: ") +
                KERNELS[i]);
      return PYPDE_ERR_COMPILE;
    }
    slots[i]->aot = nullptr;
    slots[i]->jit = f;
  }
  d.sets[N].faces = d.sets[N].faces_flux[0];
  unsigned long long gp = 0;
  size_t gsz = 0;
  int cfg[11];
  if (getglob(&gp, &gsz, mod, "pypde_cfg") != 0 ||
      cudaMemcpy(cfg, (void *)gp, sizeof(cfg), cudaMemcpyDeviceToHost) !=
          cudaSuccess) {
    set_error("cannot read the compiled launch configuration");
    return PYPDE_ERR_CUDA;
  }
  d.sets[N].pred_threads = cfg[0];
  d.sets[N].pred_cpb = cfg[1];
  d.sets[N].pred_smem = (size_t)cfg[2];
  d.sets[N].newton_threads = cfg[3];
  d.sets[N].newton_cpb = cfg[4];
  d.sets[N].newton_smem = (size_t)cfg[5];
  if (cfg[6]) {
    d.sets[N].guess_smem = (size_t)cfg[7];
    d.sets[N].guess_k1 = cfg[8];
    d.sets[N].guess_no = cfg[9];
    d.sets[N].guess_feat = cfg[10];
  } else {
    d.sets[N].guess = KFunc();
    d.sets[N].kb_guess = KFunc();
  }
  d.have[N] = true;
  return PYPDE_OK;
}

int compile_system(const char *src, const char *name, int ndim, int V,
                   int has_F, int has_B, int has_S, int second_order,
                   SystemDesc **out) {
  if (ndim < 1 || ndim > 3 || V < 1 || V > 24) {
    set_error("run-time systems need 1 <= ndim <= 3 and 1 <= V <= 24");
    return PYPDE_ERR_ARG;
  }
  SystemDesc *d = new SystemDesc();
  d->name = name;
  d->ndim = ndim;
  d->V = V;
  d->has_F = has_F;
  d->has_B = has_B;
  d->has_S = has_S;
  d->second_order = second_order;
  JitInfo *ji = new JitInfo();
  ji->src = src;
  d->module = ji;
  *out = d;
  return PYPDE_OK;
}

void release_system(SystemDesc *d) {
  if (!d)
    return;
  JitInfo *ji = (JitInfo *)d->module;
  if (ji) {
    typedef int (*unload_t)(void *);
    unload_t unload = (unload_t)drv("cuModuleUnload");
    for (int n = 0; n <= MAXN; n++)
      if (ji->modules[n] && unload)
        unload(ji->modules[n]);
    delete ji;
  }
  delete d;
}

} // namespace pypde
