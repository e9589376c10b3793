// ABI version, status strings and the per-thread last-error text.
#include <atomic>
#include <cstdarg>
#include <cstdio>

#include "common.cuh"

namespace vmck {

static thread_local char g_last_error[512] = "";

void set_last_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static std::atomic<unsigned long long> g_wait_ns{2000000000ull};

unsigned long long wait_limit_ns() { return g_wait_ns.load(std::memory_order_relaxed); }

}  // namespace vmck

extern "C" int64_t vmck_launch_count(void) { return vmck::g_launches.load(); }

extern "C" int vmck_abi_version(void) { return VMCK_ABI_VERSION; }

extern "C" int vmck_set_wait_limit_ns(uint64_t ns) {
  vmck::g_wait_ns.store(ns, std::memory_order_relaxed);
  return VMCK_OK;
}

extern "C" uint64_t vmck_wait_limit_ns(void) { return vmck::g_wait_ns.load(); }

extern "C" const char *vmck_last_error(void) { return vmck::g_last_error; }

extern "C" const char *vmck_error_string(int code) {
  switch (code) {
    case VMCK_OK: return "ok";
    case VMCK_ERR_ARG: return "invalid argument";
    case VMCK_ERR_UNSUPPORTED: return "unsupported dtype or shape";
    case VMCK_ERR_CUDA: return "CUDA runtime error";
    case VMCK_ERR_LIBRARY: return "cuBLAS / cuSOLVER error";
    case VMCK_ERR_NOMEM: return "workspace allocation failed";
    default: return "unknown status";
  }
}
