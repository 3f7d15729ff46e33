// Convolution pass kernels compiled at run time for one axis length.
//
// The 8-line y and x passes (k_fft_strided) take the axis length, and with it
// every stage's radix, column count and span, as run-time values: each shared
// memory access of a butterfly needs its address computed.  For a given axis
// length this file generates the same pass with all of them as constants
// (tile_stage_c / last_stage_c of fft_dev.cuh), compiles it with NVRTC for the
// current device and loads it with the driver API.  Every butterfly performs the
// same operations as in the library's own pass, so the results are the same
// bits; on 448 x 336 x 245 the y pass measured 74 -> 64 us.
//
// NVRTC is opened with dlopen and the driver functions are reached through the
// runtime's driver entry points, so the library links against neither.  A pass
// is compiled by a background worker thread after its first request (about a second):
// until it is loaded, and for good when NVRTC or the driver functions are
// missing or the compilation fails, the caller runs the library's pass, whose
// bits are the same.  Kernels are kept per (CUDA context, axis length, CTAs per
// SM) for the life of the process.
#include <cuda.h>
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "fft_jit.h"

namespace svie {
namespace {

typedef struct _nvrtcProgram* NvrtcProgram;
struct Nvrtc {
  int (*create)(NvrtcProgram*, const char*, const char*, int, const char* const*, const char* const*) = nullptr;
  int (*compile)(NvrtcProgram, int, const char* const*) = nullptr;
  int (*log_size)(NvrtcProgram, size_t*) = nullptr;
  int (*log)(NvrtcProgram, char*) = nullptr;
  int (*cubin_size)(NvrtcProgram, size_t*) = nullptr;
  int (*cubin)(NvrtcProgram, char*) = nullptr;
  int (*destroy)(NvrtcProgram*) = nullptr;
  bool ok = false;
};

const Nvrtc& nvrtc() {
  static Nvrtc n;
  static std::once_flag once;
  std::call_once(once, [] {
    void* h = nullptr;
    for (const char* name : {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so"})
      if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) return;
    // the builtins library NVRTC opens at its first compilation, opened here already: then it,
    // like NVRTC, is loaded before the exit handler that stops the worker is registered, and is
    // torn down after that handler has run
    for (const char* name : {"libnvrtc-builtins.so.13.0", "libnvrtc-builtins.so",
                             "/usr/local/cuda/lib64/libnvrtc-builtins.so"})
      if (dlopen(name, RTLD_NOW | RTLD_LOCAL)) break;
    n.create = (decltype(n.create))dlsym(h, "nvrtcCreateProgram");
    n.compile = (decltype(n.compile))dlsym(h, "nvrtcCompileProgram");
    n.log_size = (decltype(n.log_size))dlsym(h, "nvrtcGetProgramLogSize");
    n.log = (decltype(n.log))dlsym(h, "nvrtcGetProgramLog");
    n.cubin_size = (decltype(n.cubin_size))dlsym(h, "nvrtcGetCUBINSize");
    n.cubin = (decltype(n.cubin))dlsym(h, "nvrtcGetCUBIN");
    n.destroy = (decltype(n.destroy))dlsym(h, "nvrtcDestroyProgram");
    n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin && n.destroy;
  });
  return n;
}

struct Driver {
  CUresult (*ctx_current)(CUcontext*) = nullptr;
  CUresult (*ctx_set)(CUcontext) = nullptr;
  CUresult (*load)(CUmodule*, const void*) = nullptr;
  CUresult (*get_function)(CUfunction*, CUmodule, const char*) = nullptr;
  CUresult (*set_attribute)(CUfunction, CUfunction_attribute, int) = nullptr;
  CUresult (*launch)(const CUlaunchConfig*, CUfunction, void**, void**) = nullptr;
  bool ok = false;
};

template <class F>
void entry(const char* name, F* fn) {
  void* f = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    *fn = (F)f;
}

const Driver& driver() {
  static Driver d;
  static std::once_flag once;
  std::call_once(once, [] {
    entry("cuCtxGetCurrent", &d.ctx_current);
    entry("cuCtxSetCurrent", &d.ctx_set);
    entry("cuModuleLoadData", &d.load);
    entry("cuModuleGetFunction", &d.get_function);
    entry("cuFuncSetAttribute", &d.set_attribute);
    entry("cuLaunchKernelEx", &d.launch);
    d.ok = d.ctx_current && d.load && d.get_function && d.set_attribute && d.launch;
  });
  return d;
}

// The directory of fft_dev.cuh: csrc/ beside the loaded libsvie.so.
std::string csrc_dir() {
  Dl_info info;
  if (!dladdr((const void*)&csrc_dir, &info) || !info.dli_fname) return "";
  std::string p(info.dli_fname);
  const size_t slash = p.rfind('/');
  return (slash == std::string::npos ? std::string(".") : p.substr(0, slash)) + "/csrc";
}

// Source of the 8-line strided pass for an axis of n positions with the given
// radix sequence (forward order): the body of k_fft_strided<8, MINB> on its
// cp.async path, with each stage unrolled at compile time.  With minb >= 4 the
// stage twiddles (both orders) are read from the plan in global memory, not
// staged in shared memory: the tile buffers alone (16 n float2) then let more
// CTAs share an SM (five y tiles of n = 336).
std::string strided_source(int n, int minb, const std::vector<int>& r) {
  const int nst = (int)r.size();
  std::string s;
  char buf[512];
  auto add = [&](const char* fmt, auto... a) {
    snprintf(buf, sizeof(buf), fmt, a...);
    s += buf;
  };
  s += "#include \"fft_dev.cuh\"\nnamespace svie {\n";
  add("extern \"C\" __global__ void __launch_bounds__(256, %d) svie_jit_strided(float2* __restrict__ data, AxisPlan P,\n",
      minb);
  s += "    long long stride, int ninner, long long outer_stride, int mode, KGeom K,\n"
       "    const uint8_t* __restrict__ slabflag, int need) {\n"
       "  pdl_wait();\n  pdl_release();\n"
       "  if (slabflag && !(__ldg(slabflag + blockIdx.y) & need)) return;\n"
       "  extern __shared__ __align__(16) float2 sm[];\n";
  add("  constexpr int LW = 8, n = %d;\n", n);
  s += "  float2* const sa = sm;\n  float2* const sb = sm + LW * n;\n"
       "  const int c0 = blockIdx.x * LW;\n  const int nl = min(LW, ninner - c0);\n"
       "  float2* base = data + (long long)blockIdx.y * outer_stride + c0;\n"
       "  for (int e = threadIdx.x; e < 4 * n; e += 256) {\n"
       "    const int row = e >> 2, part = 2 * (e & 3);\n"
       "    cp_async16(sa + row * LW + part, base + row * stride + part);\n  }\n"
       "  cp_async_commit();\n";
  const bool gtw = minb >= 4;  // stage twiddles (both orders) read from the plan
  if (gtw) {
    s += "  const float2* stw = P.stw;\n";
  } else {
    s += "  const float2* stw = stage_twiddles_to_smem(sm, LW, P);\n"
         "  if (mode == 2)\n"
         "    for (int e = threadIdx.x; e < n - 1; e += 256) sm[2 * LW * n + n + e] = __ldg(P.rstw + e);\n";
  }
  s += "  cp_async_wait<0>();\n  __syncthreads();\n";
  const char* cur = "sa";
  const char* oth = "sb";
  int p = 1;
  for (int st = 0; st + 1 < nst; ++st) {
    add("  tile_stage_c<%d, %d, %d, 8, 8, 256>(%s, %s, stw, %s);\n", r[st], n / r[st], p, cur, oth,
        st == 0 ? "mode == 1" : "false");
    std::swap(cur, oth);
    p *= r[st];
  }
  const int rl = r[nst - 1];
  add("  if (mode != 2) {\n    last_stage_c<%d, %d, 8, 8, 256>(%s, stw, %s, StoreEpi{base, stride, nl, mode != 0});\n"
      "    return;\n  }\n",
      rl, n / rl, cur, nst == 1 ? "mode == 1" : "false");
  s += gtw ? "  const float2* rstw = P.rstw;\n" : "  const float2* rstw = stw + n;\n";
  s += "  const int nyh = K.ny / 2 + 1;\n"
       "  const int y = blockIdx.y, yr = min(y, K.ny - y);\n";
  add("  last_stage_c<%d, %d, 8, 8, 256>(%s, stw, false, KEpi<8>{%s, K.kred + (long long)yr * K.nzh + c0,\n"
      "      (long long)nyh * K.nzh, n, nl});\n  __syncthreads();\n",
      rl, n / rl, cur, oth);
  if (nst == 1) {
    add("  const int c = threadIdx.x %% LW, k0 = threadIdx.x / LW;\n  if (c < nl) {\n"
        "    float2* g = base + (long long)k0 * stride + c;\n"
        "    for (int k = k0; k < n; k += 256 / LW, g += (256 / LW) * stride) {\n"
        "      const float2 v = %s[k * LW + c];\n      *g = make_float2(v.x, -v.y);\n    }\n  }\n",
        oth);
  } else {
    // the inverse in reverse radix order: its first stage was the K^ epilogue
    std::vector<int> rr(r.rbegin(), r.rend());
    const char* c2 = oth;
    const char* o2 = cur;
    int p2 = rr[0];
    for (int st = 1; st + 1 < nst; ++st) {
      add("  tile_stage_c<%d, %d, %d, 8, 8, 256>(%s, %s, rstw, false);\n", rr[st], n / rr[st], p2, c2, o2);
      std::swap(c2, o2);
      p2 *= rr[st];
    }
    add("  last_stage_c<%d, %d, 8, 8, 256>(%s, rstw, false, StoreEpi{base, stride, nl, true});\n", rr[nst - 1],
        n / rr[nst - 1], c2);
  }
  s += "}\n}  // namespace svie\n";
  return s;
}

// Source of the z passes (16 line pairs per CTA at position stride 17) for an
// axis of n positions: z_r2c_body / z_c2r_body of fft_dev.cuh with the tile
// transform's stages unrolled at compile time.
std::string z_source(int n, const std::vector<int>& r) {
  std::string s;
  char buf[512];
  s += "#include \"fft_dev.cuh\"\nnamespace svie {\nstruct JitStages {\n"
       "  SVIE_DEV float2* operator()(float2* a, float2* b, const float2* stw) const {\n";
  const char* cur = "a";
  const char* oth = "b";
  int p = 1;
  for (int st = 0; st < (int)r.size(); ++st) {
    snprintf(buf, sizeof(buf), "    tile_stage_c<%d, %d, %d, 16, 17, 256>(%s, %s, stw, false);\n", r[st], n / r[st], p,
             cur, oth);
    s += buf;
    std::swap(cur, oth);
    p *= r[st];
  }
  snprintf(buf, sizeof(buf), "    return %s;\n  }\n};\n", cur);
  s += buf;
  s += "extern \"C\" __global__ void __launch_bounds__(256) svie_jit_z_r2c(const float* __restrict__ in,\n"
       "    float2* __restrict__ out, AxisPlan P, long long nlines, int nzp, const uint8_t* __restrict__ lineflag) {\n"
       "  pdl_wait();\n  pdl_release();\n"
       "  z_r2c_body<16, 17>(in, out, P, nlines, nzp, lineflag, JitStages{});\n}\n"
       "extern \"C\" __global__ void __launch_bounds__(256) svie_jit_z_c2r(const float2* __restrict__ in,\n"
       "    float* __restrict__ out, AxisPlan P, long long nlines, int nzp, float alpha, float beta,\n"
       "    const uint8_t* __restrict__ lineflag) {\n"
       "  pdl_wait();\n  pdl_release();\n"
       "  z_c2r_body<16, 17>(in, out, P, nlines, nzp, alpha, beta, lineflag, JitStages{});\n}\n"
       "}  // namespace svie\n";
  return s;
}

// Compiles a source for the current device; the cubin, or an empty vector
// with the log in *err.
std::vector<char> compile(const std::string& src, std::string* err) {
  const Nvrtc& nv = nvrtc();
  std::vector<char> out;
  if (!nv.ok) {
    *err = "NVRTC not found";
    return out;
  }
  int dev = 0, major = 0, minor = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  const std::string arch = "-arch=sm_" + std::to_string(major * 10 + minor) + (major >= 9 ? "a" : "");
  const std::string inc = "-I" + csrc_dir();
  const char* opts[] = {arch.c_str(), "-std=c++17", inc.c_str()};
  NvrtcProgram prog = nullptr;
  if (nv.create(&prog, src.c_str(), "svie_jit_strided.cu", 0, nullptr, nullptr) != 0) {
    *err = "nvrtcCreateProgram failed";
    return out;
  }
  const int rc = nv.compile(prog, 3, opts);
  size_t ls = 0;
  nv.log_size(prog, &ls);
  std::string log(ls, '\0');
  if (ls) nv.log(prog, &log[0]);
  size_t cs = 0;
  if (rc == 0 && nv.cubin_size(prog, &cs) == 0 && cs > 0) {
    out.resize(cs);
    if (nv.cubin(prog, out.data()) != 0) out.clear();
  }
  if (out.empty()) *err = "compilation failed: " + log.substr(0, 400);
  nv.destroy(&prog);
  return out;
}

// kind 0: the strided pass (minb CTAs per SM); kind 1: the z passes (minb 0)
struct Key {
  CUcontext ctx;
  int kind, n, minb;
  bool operator<(const Key& o) const {
    return std::tie(ctx, kind, n, minb) < std::tie(o.ctx, o.kind, o.n, o.minb);
  }
};
struct Fns {
  CUfunction f[2] = {nullptr, nullptr};
  int state = 0;  // 0: compiling, 1: ready, -1: failed
};
// Allocated once and never destroyed: the worker thread may still wait on them
// while the process exits, and destroying a condition variable with a waiter
// can block the exit.
std::mutex& g_mu = *new std::mutex;
std::condition_variable& g_cv = *new std::condition_variable;
std::map<Key, Fns>& g_fn = *new std::map<Key, Fns>;

// Compiles and loads `src` in the key's context and records its kernels
// `names` (run on a background thread).
void build_module(Key key, std::string src, std::vector<std::string> names) {
  const Driver& d = driver();
  Fns fns;
  std::string err;
  bool ok = d.ctx_set && d.ctx_set(key.ctx) == CUDA_SUCCESS;
  const std::vector<char> cubin = ok ? compile(src, &err) : std::vector<char>();
  CUmodule mod = nullptr;
  ok = ok && !cubin.empty() && d.load(&mod, cubin.data()) == CUDA_SUCCESS;
  for (size_t k = 0; ok && k < names.size(); ++k) {
    ok = d.get_function(&fns.f[k], mod, names[k].c_str()) == CUDA_SUCCESS &&
         d.set_attribute(fns.f[k], CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, 227 * 1024) == CUDA_SUCCESS;
    // all of the unified L1/shared storage as shared memory, for as many resident tiles as fit
    if (ok) d.set_attribute(fns.f[k], CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, 100);
  }
  if (!ok) {
    fns = Fns();
    fprintf(stderr, "[svie] fft jit: no pass for n = %d (%s); the library's pass is used\n", key.n,
            err.empty() ? "context or module load failed" : err.c_str());
  }
  fns.state = ok ? 1 : -1;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    g_fn[key] = fns;
  }
  g_cv.notify_all();
}

// One background worker compiles the requested modules in turn (a served
// stream may request many axis lengths at once; one core compiles them).  It
// exits when idle for a moment and the next request starts a new one.
// stop_worker drops the queued jobs, waits (bounded) for the compilation in
// progress and joins the worker, so that no thread of this library runs while
// the libraries are torn down.  It must run before NVRTC's own teardown: the
// exit handler registered here runs after the handlers of everything NVRTC
// initialises during its first compilation, so a host calls svie_conv_jit_stop
// on its exit path first (the Python package does so at interpreter exit).
struct Job {
  Key key;
  std::string src;
  std::vector<std::string> names;
};
std::deque<Job>& g_jobs = *new std::deque<Job>;
std::thread& g_thread = *new std::thread;  // the worker (never destroyed, like the objects above)
bool g_worker = false;   // a worker thread runs its loop (under g_mu)
bool g_busy = false;     // it is compiling (under g_mu)
bool g_stop = false;     // the process is exiting (under g_mu)

void stop_worker() {
  std::unique_lock<std::mutex> lock(g_mu);
  g_stop = true;
  g_jobs.clear();
  g_cv.notify_all();
  // the worker leaves its loop as soon as it is not compiling
  const bool left = g_cv.wait_for(lock, std::chrono::seconds(10), [] { return !g_worker; });
  lock.unlock();
  if (g_thread.joinable()) {
    if (left) g_thread.join();
    else g_thread.detach();  // still inside a compilation after 10 s: left behind
  }
}

void worker() {
  for (;;) {
    Job job;
    {
      std::unique_lock<std::mutex> lock(g_mu);
      if (!g_cv.wait_for(lock, std::chrono::milliseconds(200), [] { return g_stop || !g_jobs.empty(); }) || g_stop) {
        g_worker = false;
        lock.unlock();
        g_cv.notify_all();
        return;
      }
      job = std::move(g_jobs.front());
      g_jobs.pop_front();
      g_busy = true;
    }
    build_module(job.key, std::move(job.src), std::move(job.names));
    {
      std::lock_guard<std::mutex> lock(g_mu);
      g_busy = false;
    }
    g_cv.notify_all();
  }
}

// The kernels of a key when they are ready (SVIE_OK).  The first request
// queues their compilation for the background worker and, like every request
// until it is loaded, returns SVIE_ERR_UNSUPPORTED at once (the caller runs the
// library's pass meanwhile); a failed compilation stays failed.
int jit_get(const Key& key, const std::string& src, const std::vector<std::string>& names, CUfunction* out) {
  std::unique_lock<std::mutex> lock(g_mu);
  auto it = g_fn.find(key);
  if (it == g_fn.end()) {
    if (g_stop) return SVIE_ERR_UNSUPPORTED;
    g_fn.emplace(key, Fns());
    g_jobs.push_back(Job{key, src, names});
    if (!g_worker) {
      static bool registered = false;
      if (!registered) {
        // NVRTC and its builtins are opened first, so that this handler (the fallback of
        // svie_conv_jit_stop) runs before those libraries are torn down
        nvrtc();
        std::atexit(stop_worker);
        registered = true;
      }
      // a worker that left its loop when idle has returned or is returning (it needs no lock)
      if (g_thread.joinable()) g_thread.join();
      g_worker = true;
      g_thread = std::thread(worker);
    }
    lock.unlock();
    g_cv.notify_all();
    return SVIE_ERR_UNSUPPORTED;
  }
  if (it->second.state != 1) return SVIE_ERR_UNSUPPORTED;
  for (size_t k = 0; k < names.size(); ++k) out[k] = it->second.f[k];
  return SVIE_OK;
}

std::vector<int> radix_list(unsigned long long radices, int nst) {
  std::vector<int> r;
  for (int st = 0; st < nst; ++st) r.push_back((int)((radices >> (4 * st)) & 15ULL));
  return r;
}

bool current_context(CUcontext* ctx) {
  const Driver& d = driver();
  if (!d.ok) {
    set_error("fft jit: driver entry points not found");
    return false;
  }
  if (d.ctx_current(ctx) != CUDA_SUCCESS || !*ctx) {
    set_error("fft jit: no current CUDA context");
    return false;
  }
  return true;
}

}  // namespace

int jit_strided(int n, int minb, unsigned long long radices, int nst, CUfunction* fn) {
  *fn = nullptr;
  CUcontext ctx = nullptr;
  if (!current_context(&ctx)) return SVIE_ERR_UNSUPPORTED;
  const Key key{ctx, 0, n, minb};
  {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_fn.find(key);
    if (it != g_fn.end()) {
      if (it->second.state != 1) return SVIE_ERR_UNSUPPORTED;
      *fn = it->second.f[0];
      return SVIE_OK;
    }
  }
  return jit_get(key, strided_source(n, minb, radix_list(radices, nst)), {"svie_jit_strided"}, fn);
}

int jit_z(int n, unsigned long long radices, int nst, CUfunction* r2c, CUfunction* c2r) {
  *r2c = *c2r = nullptr;
  CUcontext ctx = nullptr;
  if (!current_context(&ctx)) return SVIE_ERR_UNSUPPORTED;
  const Key key{ctx, 1, n, 0};
  CUfunction f[2] = {nullptr, nullptr};
  int st = SVIE_ERR_UNSUPPORTED;
  bool known = false;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_fn.find(key);
    if (it != g_fn.end()) {
      known = true;
      if (it->second.state == 1) {
        f[0] = it->second.f[0];
        f[1] = it->second.f[1];
        st = SVIE_OK;
      }
    }
  }
  if (!known) st = jit_get(key, z_source(n, radix_list(radices, nst)), {"svie_jit_z_r2c", "svie_jit_z_c2r"}, f);
  *r2c = f[0];
  *c2r = f[1];
  return st;
}

bool jit_available() { return nvrtc().ok && driver().ok; }

void jit_stop() { stop_worker(); }

int jit_wait(int timeout_ms) {
  std::unique_lock<std::mutex> lock(g_mu);
  const bool done = g_cv.wait_for(lock, std::chrono::milliseconds(timeout_ms), [] {
    for (const auto& kv : g_fn)
      if (kv.second.state == 0) return false;
    return true;
  });
  return done ? SVIE_OK : SVIE_ERR_LAUNCH;
}

bool jit_launch(CUfunction fn, dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool chained, void** args) {
  const Driver& d = driver();
  CUlaunchAttribute attr[1];
  attr[0].id = CU_LAUNCH_ATTRIBUTE_PROGRAMMATIC_STREAM_SERIALIZATION;
  attr[0].value.programmaticStreamSerializationAllowed = 1;
  CUlaunchConfig cfg = {};
  cfg.gridDimX = grid.x;
  cfg.gridDimY = grid.y;
  cfg.gridDimZ = grid.z;
  cfg.blockDimX = block.x;
  cfg.blockDimY = block.y;
  cfg.blockDimZ = block.z;
  cfg.sharedMemBytes = (unsigned int)smem;
  cfg.hStream = (CUstream)s;
  cfg.attrs = attr;
  cfg.numAttrs = chained && pdl_enabled() ? 1 : 0;
  return d.ok && d.launch(&cfg, fn, args, nullptr) == CUDA_SUCCESS;
}

std::string jit_strided_source_for_test(int n, int minb, unsigned long long radices, int nst) {
  return strided_source(n, minb, radix_list(radices, nst));
}

std::string jit_z_source_for_test(int n, unsigned long long radices, int nst) {
  return z_source(n, radix_list(radices, nst));
}

}  // namespace svie
