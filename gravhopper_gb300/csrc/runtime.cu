// Library runtime: last-error capture, launch counter, device info and the
// grow-only device workspace.
#include <stdarg.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <utility>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "gh_common.cuh"

namespace gh {

// NVTX ranges, off by default (gh_trace).  The ranges are per host thread; a range is
// pushed and popped on the same thread by the Trace guard.
static std::atomic<bool> g_trace{false};
static thread_local int g_trace_depth = 0;

void trace_push(const char* name) {
  if (!g_trace.load(std::memory_order_relaxed)) return;
  nvtxRangePushA(name);
  g_trace_depth++;
}

void trace_pop() {
  if (g_trace_depth == 0) return;  // tracing was off when this scope opened
  nvtxRangePop();
  g_trace_depth--;
}

static thread_local char g_last_error[1024] = "";
static std::atomic<long long> g_launches{0};

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

void clear_error() { g_last_error[0] = '\0'; }

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Event pairs recorded around force-kernel launches while timing is enabled.
static std::mutex g_prof_mu;
static bool g_prof_on = false;
static std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_prof;
static cudaEvent_t g_prof_open = nullptr;

void prof_begin(cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (!g_prof_on) return;
  if (cudaEventCreate(&g_prof_open) != cudaSuccess) {
    g_prof_open = nullptr;
    return;
  }
  cudaEventRecord(g_prof_open, st);
}

void prof_end(cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (!g_prof_on || !g_prof_open) return;
  cudaEvent_t e1;
  if (cudaEventCreate(&e1) != cudaSuccess) return;
  cudaEventRecord(e1, st);
  g_prof.emplace_back(g_prof_open, e1);
  g_prof_open = nullptr;
}

// Pending injected faults, by kind (GH_INJECT_*).
static std::atomic<long long> g_inject[3];

bool inject_take(int fault) {
  if (fault < 1 || fault > 2) return false;
  long long k = g_inject[fault].load(std::memory_order_relaxed);
  while (k > 0)
    if (g_inject[fault].compare_exchange_weak(k, k - 1)) return true;
  return false;
}

int ensure(Buffer& b, size_t bytes) {
  if (bytes && inject_take(GH_INJECT_ALLOC)) {
    // as a growth whose cudaMalloc ran out of memory: the old buffer is gone too
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    return set_error(GH_ERR_OOM, "cudaMalloc(%zu bytes): out of memory (injected)", bytes);
  }
  if (b.bytes >= bytes && b.ptr) return GH_OK;
  if (b.ptr) {
    cudaError_t e = cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    if (e != cudaSuccess) return set_error(GH_ERR_CUDA, "cudaFree: %s", cudaGetErrorString(e));
  }
  if (bytes == 0) return GH_OK;
  // Round up so that small growth does not reallocate every call.
  size_t want = bytes + bytes / 8 + 256;
  cudaError_t e = cudaMalloc(&b.ptr, want);
  if (e != cudaSuccess) {
    b.ptr = nullptr;
    (void)cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? GH_ERR_OOM : GH_ERR_CUDA,
                     "cudaMalloc(%zu bytes): %s", want, cudaGetErrorString(e));
  }
  b.bytes = want;
  return GH_OK;
}

int device_info(DeviceInfo* out) {
  // Filled once per device under a lock: callers hold different engine locks, or none.
  static DeviceInfo cache[64];
  static std::mutex mu;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(GH_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return set_error(GH_ERR_NO_DEVICE, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lk(mu);
  if (cache[dev].device != dev) {
    DeviceInfo d;
    d.device = dev;
    GH_CUDA_TRY(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev));
    GH_CUDA_TRY(cudaDeviceGetAttribute(&d.cc_major, cudaDevAttrComputeCapabilityMajor, dev));
    GH_CUDA_TRY(cudaDeviceGetAttribute(&d.cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
    cache[dev] = d;
  }
  *out = cache[dev];
  return GH_OK;
}

}  // namespace gh

extern "C" {

const char* gh_last_error(void) { return gh::g_last_error; }

int gh_version(void) { return GH_VERSION; }

int64_t gh_launch_count(void) { return (int64_t)gh::g_launches.load(); }

int gh_trace(int enable) {
  gh::clear_error();
  gh::g_trace.store(enable != 0);
  return GH_OK;
}

int gh_debug_inject(int fault, int64_t count) {
  gh::clear_error();
  if (fault != GH_INJECT_ALLOC && fault != GH_INJECT_TREE_WAIT)
    return gh::set_error(GH_ERR_ARG, "unknown fault kind %d", fault);
  if (count < 0) return gh::set_error(GH_ERR_ARG, "negative fault count");
  gh::g_inject[fault].store(count);
  return GH_OK;
}

int gh_kernel_timing(int enable) {
  std::lock_guard<std::mutex> lk(gh::g_prof_mu);
  gh::g_prof_on = enable != 0;
  return GH_OK;
}

int gh_kernel_timing_collect(double* total_ms, int64_t* launches) {
  using namespace gh;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
  {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    ev.swap(g_prof);
  }
  double sum = 0.0;
  int rc = GH_OK;
  for (auto& p : ev) {
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(p.second);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, p.first, p.second);
    if (e != cudaSuccess && rc == GH_OK)
      rc = set_error(GH_ERR_CUDA, "kernel timing: %s", cudaGetErrorString(e));
    sum += ms;
    cudaEventDestroy(p.first);
    cudaEventDestroy(p.second);
  }
  if (total_ms) *total_ms = sum;
  if (launches) *launches = (int64_t)ev.size();
  return rc;
}

}  // extern "C"
