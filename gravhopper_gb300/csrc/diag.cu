// Throughput probes used as roofline denominators, timed with CUDA events on the
// current device: FP32 FMA (f32x2 packed) and FP64 FMA lane-operations per second,
// and the L2 read bandwidth for a buffer that stays resident in L2; and a self-check
// of the integer-pipe FP64 inverse cube against the native IEEE operations.
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

// Self-check of the integer-pipe inverse cube (f64emu.cuh) on this device: n seeded
// inputs, half with uniform significand and exponent over [2^-723, 2^727), half of
// the form dx^2 + dy^2 + dz^2 + eps^2 met by the direct sum, each compared bit for
// bit with the native RN(RN(1/s) / RN(sqrt(s))); the second half also through the
// integer-pipe squared distance (pair_inv_cube_rn from the signed components).
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ double unit_from(uint64_t r) { return (double)(r >> 11) * 0x1p-53; }

__global__ void __launch_bounds__(256)
    inv_cube_check_kernel(int64_t n, uint64_t seed, unsigned long long* counts) {
  unsigned long long wrong = 0, fallback = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t r0 = splitmix64(seed + 2 * (uint64_t)i), r1 = splitmix64(seed + 2 * (uint64_t)i + 1);
    double s, pair_d[3] = {0.0, 0.0, 0.0}, pair_eps2 = 0.0;
    if (i & 1) {
      s = __longlong_as_double(
          (long long)((r0 & 0x000FFFFFFFFFFFFFull) | ((uint64_t)(300 + (r1 >> 52) % 1450) << 52)));
    } else {
      const double dx = ldexp(unit_from(r0) - 0.5, -(int)(r1 & 31));
      const double dy = ldexp(unit_from(r1) - 0.5, -(int)((r0 >> 5) & 31));
      const double dz = unit_from(r0 ^ r1) * 0x1p-7;
      const double eps = 5e-5 * (double)(r1 % 3);
      pair_eps2 = dmul(eps, eps);
      s = dadd(dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz)), pair_eps2);
      pair_d[0] = (r0 & 1) ? -dx : dx;
      pair_d[1] = (r0 & 2) ? -dy : dy;
      pair_d[2] = (r0 & 4) ? -dz : dz;
    }
    const double want = ddiv(ddiv(1.0, s), dsqrt(s));
    double got;
    const int E = (int)((uint64_t)__double_as_longlong(s) >> 52);
    if (emu::inv_cube_rn(s, got)) {
      wrong += __double_as_longlong(got) != __double_as_longlong(want);
    } else {
      fallback += E >= 446 && E <= 1624;
    }
    if (!(i & 1)) {  // the same factor from the components, squared distance included
      int eE;
      uint64_t eM;
      emu::unpack_eps2(pair_eps2, eE, eM);
      if (emu::pair_inv_cube_rn(pair_d[0], pair_d[1], pair_d[2], eE, eM, got))
        wrong += __double_as_longlong(got) != __double_as_longlong(want);
      else
        fallback += pair_d[0] != 0.0 && pair_d[1] != 0.0 && pair_d[2] != 0.0;
    }
  }
  for (int o = 16; o; o >>= 1) {
    wrong += __shfl_xor_sync(0xffffffffu, wrong, o);
    fallback += __shfl_xor_sync(0xffffffffu, fallback, o);
  }
  if ((threadIdx.x & 31) == 0 && (wrong || fallback)) {
    atomicAdd(&counts[0], wrong);
    atomicAdd(&counts[1], fallback);
  }
}

// The mixed direct sum's pair arithmetic with every operand in registers: per pair 3
// subtractions, 3 FMAs for r^2 + eps^2, one MUFU rsqrt, 3 multiplies and 3 FMAs into
// the accumulators (12 FMA-pipe instructions and one MUFU; EQ, the equal-mass loop: 2
// multiplies, 11 instructions), MIX_R targets per thread, the "source" rotated through
// registers; no memory in the loop.  Its pairs per second are the ceiling that mix
// reaches on this GPU, below the pure FMA-chain peak.
constexpr int MIX_THREADS = 512, MIX_R = 4, MIX_UNROLL = 4;

template <bool EQ>
__global__ void __launch_bounds__(MIX_THREADS, 1) pair_mix_kernel(int iters, float seed, float* out) {
  float sx[MIX_R], sy[MIX_R], sz[MIX_R], ax[MIX_R], ay[MIX_R], az[MIX_R];
#pragma unroll
  for (int r = 0; r < MIX_R; r++) {
    sx[r] = seed * (threadIdx.x + r);
    sy[r] = seed * ((float)threadIdx.x - r);
    sz[r] = seed * (r + 1);
    ax[r] = ay[r] = az[r] = 0.f;
  }
  float4 a = make_float4(seed, 2.f * seed, 3.f * seed, 1.f);
  const float e2 = 1e-6f;
  for (int k = 0; k < iters; k++) {
#pragma unroll
    for (int u = 0; u < MIX_UNROLL; u++) {
#pragma unroll
      for (int r = 0; r < MIX_R; r++) {
        const float dx = a.x - sx[r], dy = a.y - sy[r], dz = a.z - sz[r];
        const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, e2)));
        const float ri = rsqrt_approx(r2);
        const float sc = EQ ? ri * (ri * ri) : (a.w * ri) * (ri * ri);
        ax[r] = fmaf(sc, dx, ax[r]);
        ay[r] = fmaf(sc, dy, ay[r]);
        az[r] = fmaf(sc, dz, az[r]);
      }
      a = make_float4(a.y, a.z, a.x + 1e-3f, a.w);  // the next source
    }
  }
  float s = 0.f;
#pragma unroll
  for (int r = 0; r < MIX_R; r++) s += ax[r] + ay[r] + az[r];
  if (s == 12345.678f) out[0] = s;
}

}  // namespace gh

extern "C" int gh_measure_pair_mix(int equal_mass, double* pairs_per_s, void* stream) {
  using namespace gh;
  clear_error();
  if (!pairs_per_s) return set_error(GH_ERR_ARG, "pair mix: null output");
  cudaStream_t st = (cudaStream_t)stream;
  DeviceInfo di;
  GH_TRY(device_info(&di));
  static Buffer sink;
  GH_TRY(ensure(sink, 64));
  const int iters = 1 << 12, blocks = di.num_sms;
  cudaEvent_t e0, e1;
  GH_CUDA_TRY(cudaEventCreate(&e0));
  GH_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    GH_CUDA_TRY(cudaEventRecord(e0, st));
    if (equal_mass)
      pair_mix_kernel<true><<<blocks, MIX_THREADS, 0, st>>>(iters, 1e-3f, (float*)sink.ptr);
    else
      pair_mix_kernel<false><<<blocks, MIX_THREADS, 0, st>>>(iters, 1e-3f, (float*)sink.ptr);
    GH_LAUNCH_CHECK();
    GH_CUDA_TRY(cudaEventRecord(e1, st));
    GH_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    GH_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;  // first launch is warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *pairs_per_s = (double)blocks * MIX_THREADS * iters * MIX_UNROLL * MIX_R / (best * 1e-3);
  return GH_OK;
}

extern "C" int gh_check_inv_cube(int64_t n, uint64_t seed, long long* wrong_fallback, void* stream) {
  using namespace gh;
  clear_error();
  if (!wrong_fallback || n < 0) return set_error(GH_ERR_ARG, "inverse-cube check: bad arguments");
  DeviceInfo di;
  GH_TRY(device_info(&di));
  const cudaStream_t st = (cudaStream_t)stream;
  static Buffer counts;
  GH_TRY(ensure(counts, 2 * sizeof(unsigned long long)));
  GH_CUDA_TRY(cudaMemsetAsync(counts.ptr, 0, 2 * sizeof(unsigned long long), st));
  inv_cube_check_kernel<<<4 * di.num_sms, 256, 0, st>>>(n, seed, (unsigned long long*)counts.ptr);
  GH_LAUNCH_CHECK();
  unsigned long long h[2];
  GH_CUDA_TRY(cudaMemcpyAsync(h, counts.ptr, sizeof(h), cudaMemcpyDeviceToHost, st));
  GH_CUDA_TRY(cudaStreamSynchronize(st));
  wrong_fallback[0] = (long long)h[0];
  wrong_fallback[1] = (long long)h[1];
  return GH_OK;
}

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
