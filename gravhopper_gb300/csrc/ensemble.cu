// Batched integration of many independent systems of uneven N in one persistent
// launch per step (mixed precision, drift-kick-drift), with the step loop replayed
// from a CUDA graph.
//
// Layout: the systems' particles are concatenated (system s owns [off_s, off_s+n_s));
// state x, v (N,3) FP64 and masses stay in the caller's buffers; the half-drifted
// FP32 sources live in two ping-pong float4 arrays.
// Work: one item per (system, tile of THREADS*2P targets), ordered by decreasing
// system size (longest work first); persistent CTAs take items from an atomic
// counter that the last CTA to leave resets for the next launch.  Each item covers
// all sources of its system, so the leapfrog epilogue runs in the same kernel.
#include <algorithm>
#include <mutex>
#include <vector>

#include "direct.cuh"
#include "engine.h"

namespace gh {

struct EnsSys {
  int64_t off;
  int n;
  float eps2;
  double dt;
  double origin[3];
  double meq;  // the system's common mass when all its masses are equal, else 0
};

template <bool GUARD, int THREADS, int P>
__global__ void __launch_bounds__(THREADS)
    ensemble_step_kernel(const float4* __restrict__ src, float4* __restrict__ src_next, double* __restrict__ x,
                         double* __restrict__ v, const double* __restrict__ mass, const EnsSys* __restrict__ sys,
                         const int2* __restrict__ items, int n_items, int* __restrict__ counter) {
  constexpr int JT = THREADS;
  constexpr int TILE = THREADS * 2 * P;
  __shared__ __align__(16) float4 tile[2 * 2 * JT];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  int buf = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(&counter[0], 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= n_items) break;
    const int2 w = items[it];
    const EnsSys S = sys[w.x];
    const int t = w.y;
    f2 tx[P], ty[P], tz[P], hx[P], hy[P], hz[P], lx[P], ly[P], lz[P];
#pragma unroll
    for (int p = 0; p < P; p++) {
      float4 q[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int local = t * TILE + (2 * p + h) * THREADS + tid;
        q[h] = local < S.n ? src[S.off + local] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      tx[p] = f2make(q[0].x, q[1].x);
      ty[p] = f2make(q[0].y, q[1].y);
      tz[p] = f2make(q[0].z, q[1].z);
      hx[p] = hy[p] = hz[p] = lx[p] = ly[p] = lz[p] = 0ull;
    }
    const f2 E2 = f2make(S.eps2, S.eps2);
    // Equal masses (as direct_mixed_kernel): full chunks sum r^-3 d, staged w is 1
    // (0 for padding) so the partial last chunk's general loop matches, and each
    // target's sum is scaled by the mass once.
    const bool eq = S.meq != 0.0;
    const double msc = eq ? S.meq : 1.0;
    // Double-buffered source chunks with a register prefetch (see direct_mixed_kernel).
    float4 pre = tid < S.n ? src[S.off + tid] : make_float4(0.f, 0.f, 0.f, 0.f);
    if (eq) pre.w = tid < S.n ? 1.f : 0.f;
    for (int c0 = 0; c0 < S.n; c0 += JT) {
      float4* tb = tile + buf * (2 * JT);
      tb[2 * tid + 0] = make_float4(pre.x, pre.x, pre.y, pre.y);
      tb[2 * tid + 1] = make_float4(pre.z, pre.z, pre.w, pre.w);
      __syncthreads();
      if (c0 + JT < S.n) {
        const int j = c0 + JT + tid;
        pre = j < S.n ? src[S.off + j] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (eq) pre.w = j < S.n ? 1.f : 0.f;
      }
      if (eq && c0 + JT <= S.n)
        mixed_chunk<GUARD, P, JT, true>(tb, tx, ty, tz, E2, hx, hy, hz, lx, ly, lz);
      else
        mixed_chunk<GUARD, P, JT>(tb, tx, ty, tz, E2, hx, hy, hz, lx, ly, lz);
      buf ^= 1;
    }
    EpiDKD epi;
    epi.x = x;
    epi.v = v;
    epi.mass = mass;
    epi.src_next = src_next;
    epi.xh_next = nullptr;
    epi.hist_x = epi.hist_v = nullptr;
    epi.origin = sys[w.x].origin;
    epi.dt = S.dt;
#pragma unroll
    for (int p = 0; p < P; p++) {
      float a[6], b[6];
      f2split(hx[p], a[0], b[0]);
      f2split(lx[p], a[1], b[1]);
      f2split(hy[p], a[2], b[2]);
      f2split(ly[p], a[3], b[3]);
      f2split(hz[p], a[4], b[4]);
      f2split(lz[p], a[5], b[5]);
      const int l0 = t * TILE + (2 * p) * THREADS + tid, l1 = l0 + THREADS;
      if (l0 < S.n)
        epi(S.off + l0, msc * ((double)a[0] + (double)a[1]), msc * ((double)a[2] + (double)a[3]),
            msc * ((double)a[4] + (double)a[5]));
      if (l1 < S.n)
        epi(S.off + l1, msc * ((double)b[0] + (double)b[1]), msc * ((double)b[2] + (double)b[3]),
            msc * ((double)b[4] + (double)b[5]));
    }
  }
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(&counter[1], 1) == (int)gridDim.x - 1) {
      counter[0] = 0;
      counter[1] = 0;
      __threadfence();
    }
  }
}

// Mass-weighted centre of each system (one block per system, fixed reduction order),
// and whether all its masses equal its first (finite, nonzero; a NaN never does).
__global__ void ensemble_origin_kernel(const double* __restrict__ x, const double* __restrict__ mass,
                                       EnsSys* __restrict__ sys) {
  __shared__ dvec4 red[256];
  EnsSys& S = sys[blockIdx.x];
  const double m0 = S.n > 0 ? mass[S.off] : 0.0;
  dvec4 a = make_dvec4(0.0, 0.0, 0.0, 0.0);
  bool ne = false;
  for (int k = threadIdx.x; k < S.n; k += 256) {
    const int64_t i = S.off + k;
    const double m = mass[i];
    ne |= !(m == m0);
    a.x += m * x[3 * i];
    a.y += m * x[3 * i + 1];
    a.z += m * x[3 * i + 2];
    a.w += m;
  }
  ne = __syncthreads_or(ne);
  if (threadIdx.x == 0) S.meq = (!ne && m0 != 0.0 && isfinite(m0)) ? m0 : 0.0;
  red[threadIdx.x] = a;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
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
    S.origin[0] = ok ? r.x / r.w : 0.0;
    S.origin[1] = ok ? r.y / r.w : 0.0;
    S.origin[2] = ok ? r.z / r.w : 0.0;
  }
}

// First half-drift of every system into the FP32 sources.
__global__ void ensemble_prepare_kernel(const double* __restrict__ x, const double* __restrict__ v,
                                        const double* __restrict__ mass, const EnsSys* __restrict__ sys,
                                        float4* __restrict__ src) {
  const EnsSys& S = sys[blockIdx.y];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < S.n; k += gridDim.x * blockDim.x) {
    const int64_t i = S.off + k;
    double h[3];
#pragma unroll
    for (int q = 0; q < 3; q++) h[q] = drift_half(x[3 * i + q], v[3 * i + q], S.dt);
    src[i] = make_float4((float)dsub(h[0], S.origin[0]), (float)dsub(h[1], S.origin[1]),
                         (float)dsub(h[2], S.origin[2]), (float)mass[i]);
  }
}

// ---------------------------------------------------------------------------
// Tile configurations the autotuner chooses from: (threads per CTA, packs per thread).
// ---------------------------------------------------------------------------
struct EnsConfig {
  int threads, packs;
};
static const EnsConfig kEnsConfigs[] = {{128, 2}, {256, 2}, {128, 4}, {64, 2}, {256, 1}, {64, 4}};
constexpr int kNumEnsConfigs = (int)(sizeof(kEnsConfigs) / sizeof(kEnsConfigs[0]));
constexpr int kDefaultEnsConfig = 0;

typedef void (*EnsKernel)(const float4*, float4*, double*, double*, const double*, const EnsSys*, const int2*,
                          int, int*);

template <bool G>
static EnsKernel ens_kernel_for(int cfg) {
  switch (cfg) {
    case 0: return ensemble_step_kernel<G, 128, 2>;
    case 1: return ensemble_step_kernel<G, 256, 2>;
    case 2: return ensemble_step_kernel<G, 128, 4>;
    case 3: return ensemble_step_kernel<G, 64, 2>;
    case 4: return ensemble_step_kernel<G, 256, 1>;
    default: return ensemble_step_kernel<G, 64, 4>;
  }
}

struct EnsWS {
  Buffer sys, items, counter, src[2];
  bool counter_zeroed = false;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
};
static EnsWS g_ens[64];
static std::mutex g_ens_mu;

int ensemble_run(double* x, double* v, const double* mass, const int64_t* h_off, int64_t nsys, const double* h_eps,
                 const double* h_dt, int64_t nsteps, int config, int use_graph, cudaStream_t st) {
  if (nsys < 0 || nsteps < 0) return set_error(GH_ERR_ARG, "negative nsys or nsteps");
  if (nsys == 0 || nsteps == 0) return GH_OK;
  if (!h_off || !h_eps || !h_dt) return set_error(GH_ERR_ARG, "null offsets/eps/dt");
  if (config < 0) config = kDefaultEnsConfig;
  if (config >= kNumEnsConfigs) return set_error(GH_ERR_ARG, "tile config %d out of range", config);
  const EnsConfig cf = kEnsConfigs[config];
  const int tile = cf.threads * 2 * cf.packs;
  std::vector<EnsSys> hs((size_t)nsys);
  std::vector<int2> items;
  bool guard = false;
  if (h_off[0] != 0) return set_error(GH_ERR_ARG, "offsets[0] must be 0");
  for (int64_t s = 0; s < nsys; s++) {
    const int64_t n = h_off[s + 1] - h_off[s];
    if (n < 0 || n > (1 << 24)) return set_error(GH_ERR_ARG, "system %lld has invalid size", (long long)s);
    if (!(h_eps[s] >= 0.0)) return set_error(GH_ERR_ARG, "system %lld: eps must be >= 0", (long long)s);
    hs[s].off = h_off[s];
    hs[s].n = (int)n;
    hs[s].eps2 = (float)(h_eps[s] * h_eps[s]);
    hs[s].dt = h_dt[s];
    hs[s].origin[0] = hs[s].origin[1] = hs[s].origin[2] = 0.0;
    hs[s].meq = 0.0;
    if (!(hs[s].eps2 > 0.f)) guard = true;
    for (int t = 0; t * tile < n; t++) items.push_back(make_int2((int)s, t));
  }
  const int64_t ntot = h_off[nsys];
  if (ntot == 0) return GH_OK;
  if (!x || !v || !mass) return set_error(GH_ERR_ARG, "null state buffer");
  // longest work first: cost of an item ~ its system's size
  std::stable_sort(items.begin(), items.end(),
                   [&](const int2& a, const int2& b) { return hs[a.x].n > hs[b.x].n; });

  std::lock_guard<std::mutex> lk(g_ens_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  EnsWS& ws = g_ens[di.device];
  if (!ws.stream) {
    GH_CUDA_TRY(cudaStreamCreateWithFlags(&ws.stream, cudaStreamNonBlocking));
    GH_CUDA_TRY(cudaEventCreateWithFlags(&ws.ev_in, cudaEventDisableTiming));
    GH_CUDA_TRY(cudaEventCreateWithFlags(&ws.ev_out, cudaEventDisableTiming));
  }
  // The work runs on a private stream (graphs cannot be captured on the legacy
  // default stream), ordered after and before the caller's stream by events.
  cudaStream_t ps = ws.stream;
  GH_CUDA_TRY(cudaEventRecord(ws.ev_in, st));
  GH_CUDA_TRY(cudaStreamWaitEvent(ps, ws.ev_in, 0));
  // From here on every return, error or not, orders the caller's stream after the
  // work already queued on the private stream (the next call reuses its buffers).
  struct Rejoin {
    cudaStream_t ps, st;
    cudaEvent_t ev;
    ~Rejoin() {
      if (cudaEventRecord(ev, ps) == cudaSuccess) cudaStreamWaitEvent(st, ev, 0);
    }
  } rejoin{ps, st, ws.ev_out};
  GH_TRY(ensure(ws.sys, hs.size() * sizeof(EnsSys)));
  GH_TRY(ensure(ws.items, items.size() * sizeof(int2)));
  GH_TRY(ensure(ws.src[0], (size_t)ntot * sizeof(float4)));
  GH_TRY(ensure(ws.src[1], (size_t)ntot * sizeof(float4)));
  if (!ws.counter_zeroed || ws.counter.bytes < 2 * sizeof(int)) {
    GH_TRY(ensure(ws.counter, 2 * sizeof(int)));
    GH_CUDA_TRY(cudaMemsetAsync(ws.counter.ptr, 0, 2 * sizeof(int), ps));
    ws.counter_zeroed = true;
  }
  GH_CUDA_TRY(cudaMemcpyAsync(ws.sys.ptr, hs.data(), hs.size() * sizeof(EnsSys), cudaMemcpyHostToDevice, ps));
  GH_CUDA_TRY(cudaMemcpyAsync(ws.items.ptr, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice, ps));
  EnsSys* dsys = (EnsSys*)ws.sys.ptr;
  ensemble_origin_kernel<<<(unsigned)nsys, 256, 0, ps>>>(x, mass, dsys);
  GH_LAUNCH_CHECK();
  ensemble_prepare_kernel<<<dim3(8, (unsigned)nsys), 256, 0, ps>>>(x, v, mass, dsys, (float4*)ws.src[0].ptr);
  GH_LAUNCH_CHECK();

  EnsKernel kern = guard ? ens_kernel_for<true>(config) : ens_kernel_for<false>(config);
  int occ = 1;
  GH_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, cf.threads, 0));
  if (occ < 1) occ = 1;
  int grid = di.num_sms * occ;
  if (grid > (int)items.size()) grid = (int)items.size();
  const int n_items = (int)items.size();
  const int2* ditems = (const int2*)ws.items.ptr;
  int* counter = (int*)ws.counter.ptr;
  // `captured`: recorded into a graph (counted per replay instead of here)
  auto launch = [&](int64_t k, cudaStream_t s, bool captured) -> int {
    const float4* a = (const float4*)ws.src[k & 1].ptr;
    float4* b = (float4*)ws.src[(k + 1) & 1].ptr;
    kern<<<grid, cf.threads, 0, s>>>(a, b, x, v, mass, dsys, ditems, n_items, counter);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(GH_ERR_CUDA, "ensemble launch: %s", cudaGetErrorString(e));
    if (!captured) count_launch();
    return GH_OK;
  };
  int64_t done = 0;
  if (use_graph && nsteps >= 4) {
    int64_t chunk = nsteps < 64 ? nsteps : 64;
    chunk &= ~(int64_t)1;  // even: every replay starts from src[0]
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    GH_CUDA_TRY(cudaStreamBeginCapture(ps, cudaStreamCaptureModeThreadLocal));
    int rc = GH_OK;
    for (int64_t k = 0; k < chunk && rc == GH_OK; k++) rc = launch(k, ps, true);
    cudaError_t ce = cudaStreamEndCapture(ps, &graph);
    if (rc != GH_OK || ce != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      (void)cudaGetLastError();
      return rc != GH_OK ? rc : set_error(GH_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    }
    ce = cudaGraphInstantiate(&exec, graph, 0);
    if (ce != cudaSuccess) {
      cudaGraphDestroy(graph);
      return set_error(GH_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    }
    for (; done + chunk <= nsteps; done += chunk) {
      ce = cudaGraphLaunch(exec, ps);
      if (ce != cudaSuccess) break;
      count_launch((int)chunk);
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return set_error(GH_ERR_CUDA, "graph launch: %s", cudaGetErrorString(ce));
  }
  prof_begin(ps);
  for (int64_t k = done; k < nsteps; k++) GH_TRY(launch(k - done, ps, false));
  prof_end(ps);
  return GH_OK;  // `rejoin` orders the caller's stream after the steps
}

int ensemble_num_configs() { return kNumEnsConfigs; }

}  // namespace gh
