// Throughput probes used as roofline denominators, timed with CUDA events on the
// current device: FP32 FMA (f32x2 packed) and FP64 FMA lane-operations per second,
// and the L2 read bandwidth for a buffer that stays resident in L2.
#include "direct.cuh"
#include "gh_common.cuh"

namespace gh {

constexpr int PEAK_THREADS = 256;
constexpr int PEAK_CHAINS = 8;

// Each thread runs PEAK_CHAINS independent f32x2 FMA chains: 2 FMA lane-ops per
// instruction.  The result is stored so the chains cannot be removed.
__global__ void __launch_bounds__(PEAK_THREADS) fp32_peak_kernel(int iters, float seed, float* out) {
  f2 acc[PEAK_CHAINS];
  const f2 a = f2make(0.999999f, 0.999998f);
  const f2 b = f2make(seed * 1e-7f, seed * 2e-7f);
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; c++) acc[c] = f2make(threadIdx.x + c, c - (float)threadIdx.x);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; c++) acc[c] = f2fma(acc[c], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; c++) {
    float x, y;
    f2split(acc[c], x, y);
    s += x + y;
  }
  if (s == 12345.678f) out[0] = s;
}

__global__ void __launch_bounds__(PEAK_THREADS) fp64_peak_kernel(int iters, double seed, double* out) {
  double acc[PEAK_CHAINS];
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; c++) acc[c] = threadIdx.x + c;
  const double a = 0.9999999, b = seed * 1e-9;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; c++) acc[c] = fma(acc[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; c++) s += acc[c];
  if (s == 12345.678) out[0] = s;
}

static int time_kernel(bool fp64, int iters, cudaStream_t st, double* seconds, int* blocks_out) {
  DeviceInfo di;
  GH_TRY(device_info(&di));
  int occ = 1;
  if (fp64)
    GH_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fp64_peak_kernel, PEAK_THREADS, 0));
  else
    GH_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fp32_peak_kernel, PEAK_THREADS, 0));
  const int blocks = di.num_sms * (occ > 0 ? occ : 1);
  static Buffer sink;
  GH_TRY(ensure(sink, 64));
  cudaEvent_t e0, e1;
  GH_CUDA_TRY(cudaEventCreate(&e0));
  GH_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    GH_CUDA_TRY(cudaEventRecord(e0, st));
    if (fp64)
      fp64_peak_kernel<<<blocks, PEAK_THREADS, 0, st>>>(iters, 1.0, (double*)sink.ptr);
    else
      fp32_peak_kernel<<<blocks, PEAK_THREADS, 0, st>>>(iters, 1.0f, (float*)sink.ptr);
    GH_LAUNCH_CHECK();
    GH_CUDA_TRY(cudaEventRecord(e1, st));
    GH_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    GH_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;  // first launch is warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *seconds = best * 1e-3;
  *blocks_out = blocks;
  return GH_OK;
}

// L2 read probe: every thread streams 16-byte loads that bypass L1 (ld.global.cg)
// over a buffer far smaller than L2, the same addresses on every repetition.
constexpr int L2_THREADS = 512;

__global__ void __launch_bounds__(L2_THREADS)
    l2_read_kernel(const float4* __restrict__ buf, int64_t n4, int reps, float* out) {
  const int64_t stride = (int64_t)gridDim.x * L2_THREADS;
  float acc = 0.f;
  for (int r = 0; r < reps; r++) {
    for (int64_t i = (int64_t)blockIdx.x * L2_THREADS + threadIdx.x; i < n4; i += stride) {
      const float4 v = __ldcg(buf + i);
      acc += (v.x + v.y) + (v.z + v.w);
    }
  }
  if (acc == 12345.678f) out[0] = acc;
}

static int time_l2(int64_t bytes, int reps, cudaStream_t st, double* bytes_per_s) {
  DeviceInfo di;
  GH_TRY(device_info(&di));
  int occ = 1;
  GH_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, l2_read_kernel, L2_THREADS, 0));
  const int blocks = di.num_sms * (occ > 0 ? occ : 1);
  static Buffer buf, sink;
  GH_TRY(ensure(buf, (size_t)bytes));
  GH_TRY(ensure(sink, 64));
  GH_CUDA_TRY(cudaMemsetAsync(buf.ptr, 0, (size_t)bytes, st));
  cudaEvent_t e0, e1;
  GH_CUDA_TRY(cudaEventCreate(&e0));
  GH_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    GH_CUDA_TRY(cudaEventRecord(e0, st));
    l2_read_kernel<<<blocks, L2_THREADS, 0, st>>>((const float4*)buf.ptr, bytes / 16, reps, (float*)sink.ptr);
    GH_LAUNCH_CHECK();
    GH_CUDA_TRY(cudaEventRecord(e1, st));
    GH_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    GH_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;  // first launch brings the buffer into L2
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *bytes_per_s = (double)bytes * reps / (best * 1e-3);
  return GH_OK;
}

}  // namespace gh

extern "C" int gh_measure_l2_read(double* bytes_per_s, void* stream) {
  using namespace gh;
  clear_error();
  if (!bytes_per_s) return set_error(GH_ERR_ARG, "l2 probe: null output");
  return time_l2((int64_t)32 << 20, 64, (cudaStream_t)stream, bytes_per_s);
}

extern "C" int gh_measure_fma_peaks(double* fp32_lane_ops_per_s, double* fp64_lane_ops_per_s,
                                    void* stream) {
  using namespace gh;
  clear_error();
  cudaStream_t st = (cudaStream_t)stream;
  double sec = 0.0;
  int blocks = 0;
  if (fp32_lane_ops_per_s) {
    const int iters = 1 << 11;
    GH_TRY(time_kernel(false, iters, st, &sec, &blocks));
    const double ops = (double)blocks * PEAK_THREADS * iters * PEAK_CHAINS * 2.0;
    *fp32_lane_ops_per_s = ops / sec;
  }
  if (fp64_lane_ops_per_s) {
    const int iters = 1 << 12;
    GH_TRY(time_kernel(true, iters, st, &sec, &blocks));
    const double ops = (double)blocks * PEAK_THREADS * iters * PEAK_CHAINS;
    *fp64_lane_ops_per_s = ops / sec;
  }
  return GH_OK;
}
