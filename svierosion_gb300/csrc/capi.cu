// Error reporting and small utilities of the C ABI.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>

#include <atomic>

#include "common.cuh"

namespace svie {

static thread_local char g_err[512] = "";
static std::atomic<unsigned long long> g_launches{0};

void note_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

bool pdl_enabled() {
  static const bool on = [] {
    const char* v = getenv("SVIE_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}

__global__ void k_set_f64(double* dst, double v) { *dst = v; }

}  // namespace svie

extern "C" {

const char* svie_last_error(void) { return svie::g_err; }

int svie_version(void) { return 1; }

unsigned long long svie_launch_count(void) { return svie::g_launches.load(std::memory_order_relaxed); }

int svie_set_f64(double* dst, double value, void* stream) {
  if (!dst) {
    svie::set_error("svie_set_f64: null pointer");
    return SVIE_ERR_ARG;
  }
  svie::k_set_f64<<<1, 1, 0, (cudaStream_t)stream>>>(dst, value);
  return svie::launch_status("svie_set_f64");
}

}  // extern "C"
