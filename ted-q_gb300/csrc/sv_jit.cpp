// sv_jit.cpp -- generation, NVRTC compilation, caching and launch of the
// per-circuit specialised pass kernels (see sv_jit.h).
#include "sv_jit.h"

#include <cuda.h>
#include <dlfcn.h>
#include <nvrtc.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <sys/stat.h>
#include <unistd.h>

#include <atomic>
#include <fstream>
#include <mutex>
#include <sstream>
#include <thread>

#include "sv_kernels.cuh"
#include "sv_program.h"

namespace tedq {

// ---------------------------------------------------------------- code generation

static const char* real_of(const PassParams& P) { return P.e == 1 ? "float" : "double"; }

static void emit_gate(std::ostringstream& o, const PassParams& P, const RGate& r, const char* arr) {
  const int R = P.R;
  const char* real = real_of(P);
  char buf[256];
  auto cm = [](unsigned v) { return std::to_string(v) + "u"; };
  switch (r.kind) {
    case GK_U1:
    case GK_D1:
    case GK_RXT:
    case GK_RYT:
    case GK_PH: {
      static const char* fn[] = {"apply_u1", "apply_d1", "", "", "apply_rxt", "apply_ryt", "apply_ph"};
      snprintf(buf, sizeof buf, "  %s<%d, %d, %s>(%s, c.mats[%d], CM<%s>{});\n", fn[r.kind], r.k0, R, real, arr,
               r.mat, cm(r.cmask).c_str());
      o << buf;
      break;
    }
    case GK_X:
      snprintf(buf, sizeof buf, "  apply_x<%d, %d, %s>(%s, CM<%s>{});\n", r.k0, R, real, arr, cm(r.cmask).c_str());
      o << buf;
      break;
    case GK_H:
      snprintf(buf, sizeof buf, "  apply_h<%d, %d, %s>(%s, CM<%s>{});\n", r.k0, R, real, arr, cm(r.cmask).c_str());
      o << buf;
      break;
    case GK_RXN:
    case GK_RYN:
      snprintf(buf, sizeof buf, "  %s<%d, %d, %s>(%s, c.mats[%d]);\n", r.kind == GK_RXN ? "apply_rxn" : "apply_ryn",
               r.k0, R, real, arr, r.mat);
      o << buf;
      break;
    default: {  // GK_SWAP as three controlled bit flips
      const unsigned b0 = 1u << r.k0, b1 = 1u << r.k1;
      const int tg[3] = {r.k1, r.k0, r.k1};
      const unsigned c[3] = {r.cmask | b0, r.cmask | b1, r.cmask | b0};
      for (int i = 0; i < 3; ++i) {
        snprintf(buf, sizeof buf, "  apply_x<%d, %d, %s>(%s, CM<%s>{});\n", tg[i], R, real, arr, cm(c[i]).c_str());
        o << buf;
      }
    }
  }
}

static void emit_pass(std::ostringstream& o, const PassParams& P, int index, bool adjoint) {
  const char* real = real_of(P);
  char buf[512];
  // launch bounds: pipelined variant -- one CTA of G thread groups and G + 1
  // tile slots (pipe_layout); one tile per CTA -- as many CTAs per SM as their
  // shared memory allows while every thread may keep 128 registers
  const bool pipe = pass_pipelined(P, adjoint);
  PassParams Q = P;
  Q.pipe = 1;
  const int G = pipe ? pipe_groups(Q, adjoint) : 1;
  const int threads = G << (P.m - P.R);
  const uint32_t cta_smem = pipe ? pipe_layout(Q, G, adjoint).total
                                 : tile_dynamic_smem(P, adjoint) + tile_static_smem(P, adjoint);
  const int by_smem = (int)(kPipeSmemMax / (cta_smem + 1024));
  const int min_blocks = std::max(1, std::min(by_smem, 65536 / (threads * 128)));
  const char* pro = pipe ? "" : "_TILE";
  if (!adjoint) {
    snprintf(buf, sizeof buf,
             "extern \"C\" __global__ void __launch_bounds__(%d, %d) tedq_fwd_%d(\n"
             "    const __grid_constant__ tedq::PassParams P, cpx<%s>* __restrict__ psi,\n"
             "    const %s* __restrict__ params, int n_params, const cpx<%s>* __restrict__ init, long long n_tiles) {\n"
             "  TEDQ_FWD%s_PROLOGUE(%s, %d)\n  while (c.next()) {\n",
             threads, min_blocks, index, real, real, real, pro, real, P.R);
  } else {
    snprintf(buf, sizeof buf,
             "extern \"C\" __global__ void __launch_bounds__(%d, %d) tedq_bwd_%d(\n"
             "    const __grid_constant__ tedq::PassParams P, cpx<%s>* __restrict__ psi, cpx<%s>* __restrict__ lam,\n"
             "    const %s* __restrict__ params, int n_params, double* __restrict__ grad_acc, long long n_tiles) {\n"
             "  TEDQ_BWD%s_PROLOGUE(%s, %d)\n  while (c.next()) {\n",
             threads, min_blocks, index, real, real, real, pro, real, P.R);
  }
  o << buf;
  int var = 0;
  std::vector<std::pair<std::string, int>> pending;  // gradient partials not yet reduced
  auto flush = [&]() {
    if (pending.empty()) return;
    o << "  c.grad8(";
    for (int j = 0; j < 8; ++j)
      o << (j ? ", " : "") << (j < (int)pending.size() ? pending[j].first : std::string("(") + real + ")0");
    for (int j = 0; j < 8; ++j) o << ", " << (j < (int)pending.size() ? pending[j].second : -1);
    o << ");\n";
    pending.clear();
  };
  int kap = -1;  // last normalised matrix applied (its [2].x = scale so far)
  for (int f = 0; f < P.n_phases; ++f) {
    const Phase& ph = P.phase[f];
    const bool last = f + 1 == P.n_phases;
    if (ph.type != PH_REG) {
      if (f == 0) o << "  c.to_planar();\n";
      o << "  c.dense(" << f << ");\n";
      if (last) o << "  c.to_raw();\n";
      continue;
    }
    o << (f == 0 ? "  c.begin_first(" : "  c.begin(") << f << ");\n";
    for (int g = ph.g0; g < ph.g1; ++g) {
      const RGate& r = P.gate[g];
      if (adjoint && r.grad != GR_NONE) {
        static const char* gn[] = {"", "GR_X", "GR_Y", "GR_Z", "GR_P1"};
        const std::string v = "gv" + std::to_string(var++);
        // both states carry 1 / (scale so far): the product carries its square
        const std::string k2 = kap < 0 ? "" : " * sq(c.mats[" + std::to_string(kap) + "][2].x)";
        // the empty asm pins the partial here: otherwise the compiler may sink
        // it towards grad8 and keep old copies of both states alive
        snprintf(buf, sizeof buf,
                 "  %s %s = grad_part<%s, %d, %d, %s>(c.a, c.l, CM<%uu>{})%s;\n  asm volatile(\"\" : \"+%s\"(%s));\n",
                 real, v.c_str(), gn[r.grad], r.k0, P.R, real, (unsigned)r.cmask, k2.c_str(), P.e == 1 ? "f" : "d",
                 v.c_str());
        o << buf;
        pending.push_back({v, g});
        if (pending.size() == 8) flush();
      }
      emit_gate(o, P, r, "c.a");
      if (adjoint) emit_gate(o, P, r, "c.l");
      if (r.kind == GK_RXN || r.kind == GK_RYN) kap = r.mat;
    }
    flush();
    if (f == P.norm_phase) {
      o << "  rescale<" << (int)P.R << ">(c.a, c.mats[" << (int)P.norm_last << "][2].x);\n";
      if (adjoint) o << "  rescale<" << (int)P.R << ">(c.l, c.mats[" << (int)P.norm_last << "][2].x);\n";
      kap = -1;
    }
    const bool next_wl = !last && P.phase[f + 1].type == PH_REG && P.phase[f + 1].wlocal;
    o << (last ? "  c.end_last(" : next_wl ? "  c.end_w(" : "  c.end(") << f << ");\n";
  }
  o << "  c.finish();\n  }\n  c.close();\n}\n\n";
}

std::vector<JitSource> jit_sources(const Program& p) {
  std::vector<JitSource> out;
  auto one = [&](const PassParams& P, int i, bool adjoint) {
    std::ostringstream o;
    o << "// generated by tedq_gb300: specialised pass kernel of one compiled circuit\n"
         "#include \"sv_device.cuh\"\n"
         "using namespace tedq;\nusing namespace tedq::dev;\n\n";
    emit_pass(o, P, i, adjoint);
    out.push_back({(adjoint ? "tedq_bwd_" : "tedq_fwd_") + std::to_string(i), o.str()});
  };
  for (size_t i = 0; i < p.fwd.passes.size(); ++i) one(p.fwd.passes[i], (int)i, false);
  for (size_t i = 0; i < p.bwd.passes.size(); ++i) one(p.bwd.passes[i], (int)i, true);
  return out;
}

// ---------------------------------------------------------------- NVRTC

#include "jit_headers.inc"  // kJitHeaderNames / kJitHeaderSrc (generated by build.py)

namespace {

struct Nvrtc {
  bool ok = false;
  std::string why;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcVersion) version = nullptr;
  decltype(&nvrtcGetErrorString) errstr = nullptr;
};

Nvrtc load_nvrtc() {
  Nvrtc n;
  std::vector<std::string> cands = {"libnvrtc.so.13", "libnvrtc.so"};
  for (const char* env : {"CUDA_HOME", "CUDA_PATH"})
    if (const char* d = getenv(env)) cands.push_back(std::string(d) + "/lib64/libnvrtc.so.13");
  cands.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");
  void* h = nullptr;
  for (auto& c : cands)
    if ((h = dlopen(c.c_str(), RTLD_NOW | RTLD_LOCAL))) break;
  if (!h) {
    n.why = "libnvrtc.so.13 not found";
    return n;
  }
#define TEDQ_SYM(field, name)                                  \
  n.field = reinterpret_cast<decltype(n.field)>(dlsym(h, name)); \
  if (!n.field) {                                              \
    n.why = std::string("missing symbol ") + name;             \
    return n;                                                  \
  }
  TEDQ_SYM(create, "nvrtcCreateProgram")
  TEDQ_SYM(compile, "nvrtcCompileProgram")
  TEDQ_SYM(log_size, "nvrtcGetProgramLogSize")
  TEDQ_SYM(log, "nvrtcGetProgramLog")
  TEDQ_SYM(cubin_size, "nvrtcGetCUBINSize")
  TEDQ_SYM(cubin, "nvrtcGetCUBIN")
  TEDQ_SYM(destroy, "nvrtcDestroyProgram")
  TEDQ_SYM(version, "nvrtcVersion")
  TEDQ_SYM(errstr, "nvrtcGetErrorString")
#undef TEDQ_SYM
  n.ok = true;
  return n;
}

Nvrtc& nvrtc() {
  static Nvrtc n = load_nvrtc();
  return n;
}

uint64_t fnv1a(uint64_t h, const std::string& s) {
  for (unsigned char ch : s) {
    h ^= ch;
    h *= 1099511628211ull;
  }
  return h;
}

std::string cache_dir() {
  if (const char* d = getenv("TEDQ_GB300_CACHE")) return d;
  if (const char* home = getenv("HOME")) return std::string(home) + "/.cache/tedq_gb300";
  return "/tmp/tedq_gb300_cache";
}

void mkdirs(const std::string& path) {
  std::string cur;
  for (size_t i = 0; i < path.size(); ++i) {
    cur += path[i];
    if (path[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
  }
  mkdir(path.c_str(), 0755);
}

const char* const kOptions[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo", "-DNDEBUG"};

}  // namespace

bool jit_compile(const std::string& src, std::string& cubin, std::string& err) {
  Nvrtc& N = nvrtc();
  if (!N.ok) {
    err = "NVRTC unavailable: " + N.why;
    return false;
  }
  int major = 0, minor = 0;
  N.version(&major, &minor);
  uint64_t key = 1469598103934665603ull;
  key = fnv1a(key, src);
  for (int i = 0; i < 2; ++i) key = fnv1a(key, kJitHeaderSrc[i]);
  for (const char* opt : kOptions) key = fnv1a(key, opt);
  key = fnv1a(key, std::to_string(major) + "." + std::to_string(minor));
  char name[64];
  snprintf(name, sizeof name, "/pass_%016llx.cubin", (unsigned long long)key);
  const std::string dir = cache_dir(), path = dir + name;
  {
    std::ifstream in(path, std::ios::binary);
    if (in) {
      std::stringstream ss;
      ss << in.rdbuf();
      cubin = ss.str();
      if (!cubin.empty()) return true;
    }
  }
  if (const char* dump = getenv("TEDQ_GB300_JIT_DUMP")) {  // generated source, for inspection
    mkdirs(dump);
    std::ofstream(std::string(dump) + name + ".cu") << src;
  }
  nvrtcProgram prog;
  nvrtcResult r = N.create(&prog, src.c_str(), "tedq_passes.cu", 2, kJitHeaderSrc, kJitHeaderNames);
  if (r != NVRTC_SUCCESS) {
    err = std::string("nvrtcCreateProgram: ") + N.errstr(r);
    return false;
  }
  std::vector<const char*> opts(kOptions, kOptions + sizeof(kOptions) / sizeof(kOptions[0]));
  const bool verbose = getenv("TEDQ_GB300_JIT_VERBOSE") != nullptr;
  if (verbose) opts.push_back("--ptxas-options=-v");
  r = N.compile(prog, (int)opts.size(), opts.data());
  if (verbose && r == NVRTC_SUCCESS) {
    size_t n = 0;
    N.log_size(prog, &n);
    std::string log(n, '\0');
    if (n) N.log(prog, &log[0]);
    fprintf(stderr, "%s\n", log.c_str());
  }
  if (r != NVRTC_SUCCESS) {
    size_t n = 0;
    N.log_size(prog, &n);
    std::string log(n, '\0');
    if (n) N.log(prog, &log[0]);
    err = std::string("nvrtcCompileProgram: ") + N.errstr(r) + "\n" + log.substr(0, 4000);
    N.destroy(&prog);
    return false;
  }
  size_t sz = 0;
  N.cubin_size(prog, &sz);
  cubin.assign(sz, '\0');
  N.cubin(prog, &cubin[0]);
  N.destroy(&prog);
  mkdirs(dir);
  const std::string tmp = path + ".tmp." + std::to_string(getpid());
  {
    std::ofstream out(tmp, std::ios::binary);
    out.write(cubin.data(), (std::streamsize)cubin.size());
  }
  rename(tmp.c_str(), path.c_str());
  return true;
}

bool jit_compile_all(const std::vector<JitSource>& srcs, std::vector<std::string>& cubins, std::string& err) {
  cubins.assign(srcs.size(), std::string());
  std::vector<std::string> errs(srcs.size());
  std::atomic<size_t> next(0);
  std::atomic<bool> ok(true);
  unsigned hw = std::thread::hardware_concurrency();
  if (const char* e = getenv("TEDQ_GB300_JIT_THREADS")) hw = (unsigned)atoi(e);
  const size_t nthreads = std::max<size_t>(1, std::min<size_t>(srcs.size(), hw ? hw : 4));
  auto work = [&]() {
    for (size_t i = next++; i < srcs.size() && ok; i = next++)
      if (!jit_compile(srcs[i].src, cubins[i], errs[i])) ok = false;
  };
  std::vector<std::thread> pool;
  for (size_t t = 1; t < nthreads; ++t) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  if (!ok)
    for (size_t i = 0; i < srcs.size(); ++i)
      if (!errs[i].empty()) {
        err = srcs[i].name + ": " + errs[i];
        break;
      }
  return ok;
}

// ---------------------------------------------------------------- loading and launch
// Driver functions are reached through cudaGetDriverEntryPointByVersion, so
// the library needs no link-time dependency on libcuda.

namespace {

struct Driver {
  bool ok = false;
  std::string why;
  decltype(&cuModuleLoadData) load = nullptr;
  decltype(&cuModuleGetFunction) get = nullptr;
  decltype(&cuFuncSetAttribute) set_attr = nullptr;
  decltype(&cuFuncGetAttribute) get_attr = nullptr;
  decltype(&cuLaunchKernel) launch = nullptr;
  decltype(&cuOccupancyMaxActiveBlocksPerMultiprocessor) occupancy = nullptr;
};

template <typename F>
bool entry(const char* name, F& fn, std::string& why) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
    why = std::string("driver entry point ") + name + " unavailable";
    return false;
  }
  fn = reinterpret_cast<F>(p);
  return true;
}

Driver load_driver() {
  Driver d;
  if (!entry("cuModuleLoadData", d.load, d.why) || !entry("cuModuleGetFunction", d.get, d.why) ||
      !entry("cuFuncSetAttribute", d.set_attr, d.why) || !entry("cuFuncGetAttribute", d.get_attr, d.why) ||
      !entry("cuLaunchKernel", d.launch, d.why) ||
      !entry("cuOccupancyMaxActiveBlocksPerMultiprocessor", d.occupancy, d.why))
    return d;
  d.ok = true;
  return d;
}

Driver& driver() {
  static std::once_flag once;
  static Driver d;
  std::call_once(once, [] { d = load_driver(); });
  return d;
}

}  // namespace

bool jit_load(const std::vector<std::string>& cubins, const std::vector<JitSource>& srcs, int n_fwd, int n_bwd,
              JitKernels& out, std::string& err) {
  Driver& D = driver();
  if (!D.ok) {
    err = D.why;
    return false;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) {
    err = "no current CUDA device";
    return false;
  }
  if ((int)cubins.size() != n_fwd + n_bwd || srcs.size() != cubins.size()) {
    err = "kernel count mismatch";
    return false;
  }
  for (size_t i = 0; i < cubins.size(); ++i) {
    CUmodule mod = nullptr;
    CUresult r = D.load(&mod, cubins[i].data());
    if (r != CUDA_SUCCESS) {
      err = "cuModuleLoadData failed (" + std::to_string((int)r) + ")";
      return false;
    }
    out.modules.push_back(mod);
    CUfunction f = nullptr;
    if (D.get(&f, mod, srcs[i].name.c_str()) != CUDA_SUCCESS) {
      err = "missing kernel " + srcs[i].name;
      return false;
    }
    // dynamic shared memory up to the per-block limit left by the static part
    // (the one-tile-per-CTA variant keeps its matrices in static memory)
    int static_bytes = 0;
    if (D.get_attr(&static_bytes, CU_FUNC_ATTRIBUTE_SHARED_SIZE_BYTES, f) != CUDA_SUCCESS ||
        D.set_attr(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)kPipeSmemMax - static_bytes) !=
            CUDA_SUCCESS) {
      err = "cannot set the shared-memory limit of " + srcs[i].name;
      return false;
    }
    ((int)i < n_fwd ? out.fwd : out.bwd).push_back(reinterpret_cast<void*>(f));
  }
  return true;
}

// Driver launch results as runtime errors (a refused launch is not reported
// as a failed kernel).
static cudaError_t to_rt(CUresult r) {
  switch (r) {
    case CUDA_SUCCESS: return cudaSuccess;
    case CUDA_ERROR_INVALID_VALUE: return cudaErrorInvalidValue;
    case CUDA_ERROR_OUT_OF_MEMORY: return cudaErrorMemoryAllocation;
    case CUDA_ERROR_LAUNCH_OUT_OF_RESOURCES: return cudaErrorLaunchOutOfResources;
    case CUDA_ERROR_INVALID_HANDLE: return cudaErrorInvalidResourceHandle;
    case CUDA_ERROR_NOT_SUPPORTED: return cudaErrorNotSupported;
    default: return cudaErrorLaunchFailure;
  }
}

static cudaError_t driver_residency(const void* key, int threads, size_t smem, int* per_sm) {
  CUfunction f = reinterpret_cast<CUfunction>(const_cast<void*>(key));
  return driver().occupancy(per_sm, f, threads, smem) == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidConfiguration;
}

cudaError_t jit_launch_fwd(void* fn, bool dbl, const PassParams& P0, void* psi, const void* params, int n_params,
                           const void* init, int64_t batch, cudaStream_t s) {
  (void)dbl;
  PassParams P = P0;
  P.pipe = pass_pipelined(P0, false) ? 1 : 0;
  const int G = pipe_groups(P, false);
  const unsigned smem = P.pipe ? pipe_layout(P, G, false).total : tile_dynamic_smem(P, false),
                 T = (unsigned)G << (P.m - P.R);
  long long n_tiles = (long long)(batch << (P.n - P.m));
  CUfunction f = reinterpret_cast<CUfunction>(fn);
  unsigned grid = (unsigned)n_tiles;
  if (P.pipe) {
    cudaError_t e = pass_grid_cached(fn, (int)T, smem, n_tiles, driver_residency, grid);
    if (e != cudaSuccess) return e;
  }
  void* args[] = {const_cast<PassParams*>(&P), &psi, const_cast<void**>(&params), &n_params,
                  const_cast<void**>(&init), &n_tiles};
  return to_rt(driver().launch(f, grid, 1, 1, T, 1, 1, smem, reinterpret_cast<CUstream>(s), args, nullptr));
}

cudaError_t jit_launch_bwd(void* fn, bool dbl, const PassParams& P0, void* psi, void* lam, const void* params,
                           int n_params, double* grad_acc, int64_t batch, cudaStream_t s) {
  (void)dbl;
  PassParams P = P0;
  P.pipe = pass_pipelined(P0, true) ? 1 : 0;
  const int G = pipe_groups(P, true);
  const unsigned smem = P.pipe ? pipe_layout(P, G, true).total : tile_dynamic_smem(P, true),
                 T = (unsigned)G << (P.m - P.R);
  long long n_tiles = (long long)(batch << (P.n - P.m));
  CUfunction f = reinterpret_cast<CUfunction>(fn);
  unsigned grid = (unsigned)n_tiles;
  if (P.pipe) {
    cudaError_t e = pass_grid_cached(fn, (int)T, smem, n_tiles, driver_residency, grid);
    if (e != cudaSuccess) return e;
  }
  void* args[] = {const_cast<PassParams*>(&P), &psi, &lam, const_cast<void**>(&params), &n_params, &grad_acc,
                  &n_tiles};
  return to_rt(driver().launch(f, grid, 1, 1, T, 1, 1, smem, reinterpret_cast<CUstream>(s), args, nullptr));
}

}  // namespace tedq
