// Mixed-precision direct-sum force that allocates no device memory.
//
// Some callers cannot let a library allocate: an application that owns all device
// memory through its own pool and forbids other allocations, or a time-stepping loop
// that must not hit cudaMalloc/cudaFree because they can synchronise the device and
// stall its streams.  gh_direct_mixed_noalloc serves them: the caller passes inputs
// and outputs, and every scratch buffer the stream-K kernel needs (FP32 sources,
// per-CTA partial sums, per-tile counters, the origin) lives in one file-scope
// __device__ array of fixed size, which each GPU that loads this library holds until
// the process exits.
#include <mutex>

#include "direct.cuh"

namespace gh {

// Largest particle count accepted by the no-allocation entry point.
constexpr int64_t NOALLOC_MAX_N = 65536;
// Kernel shape: 256 threads, 2 f32x2 packs (1024 targets per tile), 2 CTAs per SM.
constexpr int NA_THREADS = 256, NA_P = 2, NA_MINB = 2;
constexpr int NA_TILE = NA_THREADS * 2 * NA_P;
// Bytes set aside for per-CTA partial sums (each CTA may leave partials for two tiles,
// its first and its last).  The persistent grid is capped by what fits: 304 CTAs, i.e.
// 2 per SM on a 152-SM GB300 (its occupancy).  A part with more SMs runs at most 304
// CTAs here; the stream-K split still gives each of them an equal share of the pairs.
constexpr size_t NA_PART_BUDGET = (size_t)304 * 2 * mixed_slot_floats(NA_THREADS, NA_P) * sizeof(float);
constexpr int64_t NA_MAX_GRID = (int64_t)(NA_PART_BUDGET / (2 * mixed_slot_floats(NA_THREADS, NA_P) * sizeof(float)));
constexpr int64_t NA_MAX_TILES = (NOALLOC_MAX_N + NA_TILE - 1) / NA_TILE;
constexpr int NA_COM_THREADS = 256;

// Byte layout of the scratch array (each region 256-byte aligned).
constexpr size_t na_align(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t NA_OFF_SRC = 0;
constexpr size_t NA_OFF_PART = NA_OFF_SRC + na_align(NOALLOC_MAX_N * sizeof(float4));
constexpr size_t NA_OFF_CNT = NA_OFF_PART + na_align(NA_PART_BUDGET);
constexpr size_t NA_OFF_ORIGIN = NA_OFF_CNT + na_align(NA_MAX_TILES * sizeof(int));
constexpr size_t NA_BYTES = NA_OFF_ORIGIN + na_align(4 * sizeof(double));  // about 16 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

// Mass-weighted centre in one block with a fixed reduction order.
__global__ void __launch_bounds__(NA_COM_THREADS)
    na_origin_kernel(const double* __restrict__ pos, const double* __restrict__ mass, int64_t n,
                     double* __restrict__ origin) {
  __shared__ dvec4 red[NA_COM_THREADS];
  dvec4 a = make_dvec4(0.0, 0.0, 0.0, 0.0);
  for (int64_t i = threadIdx.x; i < n; i += NA_COM_THREADS) {
    const double m = mass[i];
    a.x += m * pos[3 * i];
    a.y += m * pos[3 * i + 1];
    a.z += m * pos[3 * i + 2];
    a.w += m;
  }
  red[threadIdx.x] = a;
  __syncthreads();
  for (int s = NA_COM_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[threadIdx.x].x += red[threadIdx.x + s].x;
      red[threadIdx.x].y += red[threadIdx.x + s].y;
      red[threadIdx.x].z += red[threadIdx.x + s].z;
      red[threadIdx.x].w += red[threadIdx.x + s].w;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const dvec4 r = red[0];
    const bool ok = r.w != 0.0 && isfinite(r.x / r.w) && isfinite(r.y / r.w) && isfinite(r.z / r.w);
    origin[0] = ok ? r.x / r.w : 0.0;
    origin[1] = ok ? r.y / r.w : 0.0;
    origin[2] = ok ? r.z / r.w : 0.0;
  }
}

__global__ void na_sources_kernel(const double* __restrict__ pos, const double* __restrict__ mass, int64_t n,
                                  const double* __restrict__ origin, float4* __restrict__ src) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  src[i] = make_float4((float)dsub(pos[3 * i], origin[0]), (float)dsub(pos[3 * i + 1], origin[1]),
                       (float)dsub(pos[3 * i + 2], origin[2]), (float)mass[i]);
}

// Device address of the scratch array on each device.  Host code cannot use the
// array's name as a device pointer, so the address comes from cudaGetSymbolAddress
// with the device current.  It is looked up again on every call made outside stream
// capture (a lookup is cheap), so a context torn down and re-created between calls
// (cudaDeviceReset) never leaves a stale address behind; a call made during capture
// uses the address of the last uncaptured call on that device, and the first call on a
// device must come before any capture.
static unsigned char* g_na_base[64];
static std::mutex g_na_mu;

static int na_scratch(int device, cudaStream_t st, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_na_mu);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  GH_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
  if (cs == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return set_error(GH_ERR_CUDA, "cudaGetSymbolAddress(no-alloc scratch): %s", cudaGetErrorString(e));
    g_na_base[device] = (unsigned char*)p;
  } else if (!g_na_base[device]) {
    return set_error(GH_ERR_ARG, "gh_direct_mixed_noalloc: the first call on a device must not be captured");
  }
  *out = g_na_base[device];
  return GH_OK;
}

template <bool G>
static int na_occupancy() {
  int o = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, direct_mixed_kernel<G, NA_THREADS, NA_P, NA_MINB, EpiStore>,
                                                    NA_THREADS, 0) != cudaSuccess ||
      o < 1)
    o = 1;
  return o;
}

}  // namespace gh

extern "C" int gh_direct_mixed_noalloc(const double* pos, const double* mass, int64_t np, double eps, double* acc,
                                       void* stream) {
  using namespace gh;
  clear_error();
  if (np < 0) return set_error(GH_ERR_ARG, "negative particle count");
  if (np > NOALLOC_MAX_N)
    return set_error(GH_ERR_ARG, "gh_direct_mixed_noalloc: %lld particles exceed its fixed limit of %lld",
                     (long long)np, (long long)NOALLOC_MAX_N);
  if (!(eps >= 0.0)) return set_error(GH_ERR_ARG, "eps must be >= 0 (got %g)", eps);
  if (np == 0) return GH_OK;
  if (!pos || !mass || !acc) return set_error(GH_ERR_ARG, "null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  DeviceInfo di;
  GH_TRY(device_info(&di));
  unsigned char* base = nullptr;
  GH_TRY(na_scratch(di.device, st, &base));
  float4* src = (float4*)(base + NA_OFF_SRC);
  float* partials = (float*)(base + NA_OFF_PART);
  int* counters = (int*)(base + NA_OFF_CNT);
  double* origin = (double*)(base + NA_OFF_ORIGIN);

  const float eps2 = (float)(eps * eps);
  const bool guard = !(eps2 > 0.f);
  int64_t cap = (int64_t)di.num_sms * (guard ? na_occupancy<true>() : na_occupancy<false>());
  if (cap > NA_MAX_GRID) cap = NA_MAX_GRID;
  const StreamK sk = mixed_plan(np, np, cap, NA_TILE, NA_THREADS);
  // The array keeps the previous call's contents: the tile counters must start at zero.
  GH_CUDA_TRY(cudaMemsetAsync(counters, 0, (size_t)sk.n_tiles * sizeof(int), st));
  na_origin_kernel<<<1, NA_COM_THREADS, 0, st>>>(pos, mass, np, origin);
  GH_LAUNCH_CHECK();
  na_sources_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(pos, mass, np, origin, src);
  GH_LAUNCH_CHECK();
  EpiStore epi{acc};
  if (guard)
    direct_mixed_kernel<true, NA_THREADS, NA_P, NA_MINB, EpiStore>
        <<<(unsigned)sk.grid, NA_THREADS, 0, st>>>(src, np, src, np, eps2, sk, partials, counters, epi,
                                                   nullptr);
  else
    direct_mixed_kernel<false, NA_THREADS, NA_P, NA_MINB, EpiStore>
        <<<(unsigned)sk.grid, NA_THREADS, 0, st>>>(src, np, src, np, eps2, sk, partials, counters, epi,
                                                   nullptr);
  GH_LAUNCH_CHECK();
  return GH_OK;
}
