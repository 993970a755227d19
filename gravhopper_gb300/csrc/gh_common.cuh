// Shared definitions for the GB300 gravity engine: status codes, error capture,
// exact FP64 helpers, unit factors and the per-device workspace.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/gravhopper_gb300.h"

// ---------------------------------------------------------------------------
// Unit factors.  Code units are G=1, kpc, Msun (gravhopper/_jbgrav.c:137-139); the
// host works in kpc, km/s, Msun, Myr (gravhopper/gravhopper.py:146-151).
//   ACCEL_UNIT      G*Msun/kpc^2 in km/s/Myr  (gravhopper/jbgrav.py:40-48)
//   KMS_MYR_TO_KPC  (km/s)*Myr in kpc          (astropy conversion in gravhopper.py:409,416)
// ---------------------------------------------------------------------------
#define GH_ACCEL_UNIT 4.398600412921223e-09
#define GH_KMS_MYR_TO_KPC 1.022712165045695e-03

namespace gh {

// Records a formatted message as the thread's last error and returns `code`.
int set_error(int code, const char* fmt, ...);
void clear_error();

// Launch counter: every kernel launched by the library increments it (host side).
void count_launch(int n = 1);

// Optional CUDA-event timing of the dominant kernels (the force kernels), enabled by
// gh_kernel_timing(1): prof_begin/prof_end bracket one launch on its stream.
void prof_begin(cudaStream_t st);
void prof_end(cudaStream_t st);

#define GH_CUDA_TRY(expr)                                                        \
  do {                                                                           \
    cudaError_t _e = (expr);                                                     \
    if (_e != cudaSuccess)                                                       \
      return ::gh::set_error(GH_ERR_CUDA, "%s failed: %s (%s:%d)", #expr,        \
                             cudaGetErrorString(_e), __FILE__, __LINE__);        \
  } while (0)

#define GH_LAUNCH_CHECK()                                                        \
  do {                                                                           \
    ::gh::count_launch();                                                        \
    cudaError_t _e = cudaGetLastError();                                         \
    if (_e != cudaSuccess)                                                       \
      return ::gh::set_error(GH_ERR_CUDA, "kernel launch failed: %s (%s:%d)",   \
                             cudaGetErrorString(_e), __FILE__, __LINE__);        \
  } while (0)

#define GH_TRY(expr)              \
  do {                            \
    int _rc = (expr);             \
    if (_rc != GH_OK) return _rc; \
  } while (0)

// ---------------------------------------------------------------------------
// Exact (never contracted) FP64 arithmetic.  The reference is plain C compiled
// without FMA contraction on x86-64, so every a*b+c there is two roundings.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double dsqrt(double a) { return __dsqrt_rn(a); }

// 32-byte aligned 4-vector of doubles (x, y, z, w).
struct __align__(32) dvec4 {
  double x, y, z, w;
};
__host__ __device__ __forceinline__ dvec4 make_dvec4(double x, double y, double z, double w) {
  dvec4 r;
  r.x = x;
  r.y = y;
  r.z = z;
  r.w = w;
  return r;
}

// Hardware reciprocal square root (MUFU), flush-to-zero.  Inputs are >= eps^2 > 0.
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Error-free transformation (Knuth two-sum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// ---------------------------------------------------------------------------
// Device workspace: grow-only buffers owned by the library, one set per device.
// ---------------------------------------------------------------------------
struct Buffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

// Ensures `b` holds at least `bytes`; contents are not preserved on growth.
int ensure(Buffer& b, size_t bytes);

// Host-side fault injection for tests (gh_debug_inject): true, and one fewer pending,
// when a fault of this kind is pending.
bool inject_take(int fault);

// Optional NVTX ranges (gh_trace): a named range over a scope of host code, visible to
// NVTX-aware tools (Nsight Compute's --nvtx filters, Nsight Systems); no-ops while off.
void trace_push(const char* name);
void trace_pop();
struct Trace {
  explicit Trace(const char* name) { trace_push(name); }
  ~Trace() { trace_pop(); }
  Trace(const Trace&) = delete;
  Trace& operator=(const Trace&) = delete;
};

struct DeviceInfo {
  int device = -1;
  int num_sms = 0;
  int cc_major = 0, cc_minor = 0;
};
int device_info(DeviceInfo* out);

}  // namespace gh
