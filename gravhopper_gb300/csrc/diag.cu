// Pipe-throughput probes used as roofline denominators: FP32 FMA (f32x2 packed) and
// FP64 FMA lane-operations per second on the current device, timed with CUDA events.
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

}  // namespace gh

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
