// Direct-sum force calls and the on-device leapfrog run loop.
#include <mutex>

#include "direct.cuh"
#include "engine.h"

namespace gh {


// ---------------------------------------------------------------------------
// Small kernels: mass-weighted centre (deterministic two-pass), conversion to
// FP32 relative coordinates, first half-drift of a run.
// ---------------------------------------------------------------------------
constexpr int COM_THREADS = 256;
constexpr int COM_MAX_BLOCKS = 512;

// Also flags, per block, whether every mass of the block equals mass[0] (a NaN never
// does), for the mixed kernel's equal-mass loop.
__global__ void com_partial_kernel(const double* __restrict__ pos, const double* __restrict__ mass,
                                   int64_t n, dvec4* __restrict__ part, int* __restrict__ differ) {
  __shared__ dvec4 red[COM_THREADS];
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = (int64_t)blockIdx.x * per;
  const int64_t b1 = b0 + per < n ? b0 + per : n;
  const double m0 = n > 0 ? mass[0] : 0.0;
  dvec4 acc = make_dvec4(0.0, 0.0, 0.0, 0.0);
  bool ne = false;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += COM_THREADS) {
    double m = mass[i];
    ne |= !(m == m0);
    acc.x += m * pos[3 * i];
    acc.y += m * pos[3 * i + 1];
    acc.z += m * pos[3 * i + 2];
    acc.w += m;
  }
  ne = __syncthreads_or(ne);
  if (threadIdx.x == 0) differ[blockIdx.x] = ne;
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = COM_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      dvec4 o = red[threadIdx.x + s];
      red[threadIdx.x].x += o.x;
      red[threadIdx.x].y += o.y;
      red[threadIdx.x].z += o.z;
      red[threadIdx.x].w += o.w;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// origin[0..2]: the mass-weighted centre; origin[3]: the common mass of all particles
// when they share one that is finite and nonzero, else 0.
__global__ void com_final_kernel(const dvec4* __restrict__ part, const int* __restrict__ differ, int nb,
                                 const double* __restrict__ mass, int64_t n, double* __restrict__ origin) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  dvec4 s = make_dvec4(0.0, 0.0, 0.0, 0.0);
  bool ne = false;
  for (int b = 0; b < nb; b++) {
    s.x += part[b].x;
    s.y += part[b].y;
    s.z += part[b].z;
    s.w += part[b].w;
    ne |= differ[b] != 0;
  }
  const double m0 = n > 0 ? mass[0] : 0.0;
  origin[3] = (!ne && m0 != 0.0 && isfinite(m0)) ? m0 : 0.0;
  if (s.w != 0.0 && isfinite(s.x / s.w) && isfinite(s.y / s.w) && isfinite(s.z / s.w)) {
    origin[0] = s.x / s.w;
    origin[1] = s.y / s.w;
    origin[2] = s.z / s.w;
  } else {
    origin[0] = origin[1] = origin[2] = 0.0;
  }
}

__global__ void to_f32_kernel(const double* __restrict__ pos, const double* __restrict__ mass,
                              int64_t n, const double* __restrict__ origin, float4* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double o0 = origin[0], o1 = origin[1], o2 = origin[2];
  out[i] = make_float4((float)dsub(pos[3 * i], o0), (float)dsub(pos[3 * i + 1], o1),
                       (float)dsub(pos[3 * i + 2], o2), mass ? (float)mass[i] : 0.f);
}

__global__ void drift_prepare_kernel(const double* __restrict__ x, const double* __restrict__ v,
                                     const double* __restrict__ mass, int64_t n, double dt,
                                     const double* __restrict__ origin, float4* __restrict__ src,
                                     double* __restrict__ xh) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double h[3];
#pragma unroll
  for (int k = 0; k < 3; k++) h[k] = drift_half(x[3 * i + k], v[3 * i + k], dt);
  if (src)
    src[i] = make_float4((float)dsub(h[0], origin[0]), (float)dsub(h[1], origin[1]),
                         (float)dsub(h[2], origin[2]), (float)mass[i]);
  if (xh) {
#pragma unroll
    for (int k = 0; k < 3; k++) xh[3 * i + k] = h[k];
  }
}

// ---------------------------------------------------------------------------
// Workspace for the direct path (one per device).
// ---------------------------------------------------------------------------
struct DirectWS {
  Buffer src[2], tgt, xh[2], partials, counters, origin, com_part;
  size_t counters_zeroed = 0;
};
static DirectWS g_ws[64];
static std::recursive_mutex g_mu;

// Shape of the mixed kernel (index into kMixedShapes); -1 picks by problem size.
static int g_mixed_shape = -1;
static int g_f64_form = -1;  // -1 by target count, 0 thread per target, 1 ordered CTA-wide terms

// Chosen from a sweep of the shapes on GB300 (force and fused leapfrog step, N = 2048
// to 1M): small systems want small tiles (more CTAs share the sources); from N ~ 24k
// the scalar FP32 loop with wide CTAs wins, 512 threads x 4 targets for a force at
// every size (e.g. 1.78 ms against 1.93 ms for the packed 128 x 4 at N = 65,536) and
// for the leapfrog step up to ~128k, 384 threads x 6 targets for larger steps, whose
// heavier epilogue favours it (435 ms per step at N = 1M against 443 ms).
//
// An autotuner can replace that table (gh_direct_tune): per epilogue kind (force or
// fused leapfrog step), rules "from n_min particles on, shape k"; the rule with the
// largest n_min <= n applies, and sizes below every rule fall back to the table.
constexpr int kMaxTuneRules = 32;
struct TuneRule {
  int64_t n_min;
  int shape;
};
static TuneRule g_tune[2][kMaxTuneRules];
static int g_ntune[2] = {0, 0};
static std::mutex g_tune_mu;

static int tuned_shape(int64_t n, bool dkd) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  const int k = dkd ? 1 : 0;
  int best = -1;
  int64_t best_min = -1;
  for (int r = 0; r < g_ntune[k]; r++)
    if (g_tune[k][r].n_min <= n && g_tune[k][r].n_min > best_min) {
      best_min = g_tune[k][r].n_min;
      best = g_tune[k][r].shape;
    }
  return best;
}

static int auto_shape(int64_t np, int64_t nt, bool dkd) {
  const int64_t n = np > nt ? np : nt;
  const int tuned = tuned_shape(n, dkd);
  if (tuned >= 0) return tuned;
  if (n < 12288) return 7;                   // packed, 256 threads, 1 pack, 4 CTAs/SM
  if (n < 24576) return 3;                   // packed, 128 threads, 2 packs, 4 CTAs/SM
  if (dkd && n >= (1 << 17)) return 12;      // scalar, 384 threads x 6 targets
  return 10;                                 // scalar, 512 threads x 4 targets
}

template <bool G, int T, int P, int B, class Epi, bool PK = true>
static int launch_shape(const StreamK& sk, const float4* src, int64_t np, const float4* tgt, int64_t nt,
                        float eps2, float* partials, int* counters, const Epi& epi, const double* eqm,
                        cudaStream_t st) {
  direct_mixed_kernel<G, T, P, B, Epi, PK><<<(unsigned)sk.grid, T, 0, st>>>(src, np, tgt, nt, eps2, sk, partials,
                                                                            counters, epi, eqm);
  return GH_OK;
}

template <bool G, int T, int P, int B, bool PK = true>
static int occupancy_shape() {
  int o = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, direct_mixed_kernel<G, T, P, B, EpiStore, PK>, T, 0) !=
          cudaSuccess ||
      o < 1)
    o = 1;
  return o;
}

template <bool G, class Epi>
static int dispatch_shape(int shape, const StreamK& sk, const float4* src, int64_t np, const float4* tgt,
                          int64_t nt, float eps2, float* partials, int* counters, const Epi& epi,
                          const double* eqm, cudaStream_t st) {
  switch (shape) {
    case 0: return launch_shape<G, 256, 2, 2>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 1: return launch_shape<G, 256, 4, 1>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 2: return launch_shape<G, 128, 4, 2>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 3: return launch_shape<G, 128, 2, 4>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 4: return launch_shape<G, 512, 2, 1>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 5: return launch_shape<G, 256, 2, 3>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 6: return launch_shape<G, 128, 2, 6>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 7: return launch_shape<G, 256, 1, 4>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 8: return launch_shape<G, 512, 2, 2>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 9: return launch_shape<G, 256, 2, 2, Epi, false>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 10: return launch_shape<G, 512, 2, 1, Epi, false>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    case 11: return launch_shape<G, 256, 4, 1, Epi, false>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
    default: return launch_shape<G, 384, 3, 1, Epi, false>(sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
  }
}

static int mixed_grid_cap(int num_sms, int shape, bool guard) {
  static int occ[2][kNumMixedShapes] = {};
  int& o = occ[guard ? 1 : 0][shape];
  if (o == 0) {
    switch (shape) {
      case 0: o = guard ? occupancy_shape<true, 256, 2, 2>() : occupancy_shape<false, 256, 2, 2>(); break;
      case 1: o = guard ? occupancy_shape<true, 256, 4, 1>() : occupancy_shape<false, 256, 4, 1>(); break;
      case 2: o = guard ? occupancy_shape<true, 128, 4, 2>() : occupancy_shape<false, 128, 4, 2>(); break;
      case 3: o = guard ? occupancy_shape<true, 128, 2, 4>() : occupancy_shape<false, 128, 2, 4>(); break;
      case 4: o = guard ? occupancy_shape<true, 512, 2, 1>() : occupancy_shape<false, 512, 2, 1>(); break;
      case 5: o = guard ? occupancy_shape<true, 256, 2, 3>() : occupancy_shape<false, 256, 2, 3>(); break;
      case 6: o = guard ? occupancy_shape<true, 128, 2, 6>() : occupancy_shape<false, 128, 2, 6>(); break;
      case 7: o = guard ? occupancy_shape<true, 256, 1, 4>() : occupancy_shape<false, 256, 1, 4>(); break;
      case 8: o = guard ? occupancy_shape<true, 512, 2, 2>() : occupancy_shape<false, 512, 2, 2>(); break;
      case 9: o = guard ? occupancy_shape<true, 256, 2, 2, false>() : occupancy_shape<false, 256, 2, 2, false>(); break;
      case 10:
        o = guard ? occupancy_shape<true, 512, 2, 1, false>() : occupancy_shape<false, 512, 2, 1, false>();
        break;
      case 11:
        o = guard ? occupancy_shape<true, 256, 4, 1, false>() : occupancy_shape<false, 256, 4, 1, false>();
        break;
      default:
        o = guard ? occupancy_shape<true, 384, 3, 1, false>() : occupancy_shape<false, 384, 3, 1, false>();
        break;
    }
  }
  return o * num_sms;
}

StreamK mixed_plan(int64_t np, int64_t nt, int64_t grid_cap, int tile, int jt) {
  StreamK s;
  s.n_tiles = (nt + tile - 1) / tile;
  s.chunks = (np + jt - 1) / jt;
  s.units = s.n_tiles * s.chunks;
  s.grid = s.units < grid_cap ? s.units : grid_cap;
  if (s.grid < 1) s.grid = 1;
  return s;
}

int set_f64_form(int form) {
  if (form < -1 || form > 1) return set_error(GH_ERR_ARG, "fp64 form %d out of range", form);
  g_f64_form = form;
  return GH_OK;
}

int tune_rule(int64_t n_min, int fused_step, int shape) {
  if (fused_step != 0 && fused_step != 1) return set_error(GH_ERR_ARG, "fused_step must be 0 or 1");
  if (shape >= kNumMixedShapes) return set_error(GH_ERR_ARG, "mixed shape %d out of range", shape);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (shape < 0) {  // clear this kind's rules
    g_ntune[fused_step] = 0;
    return GH_OK;
  }
  if (n_min < 0) return set_error(GH_ERR_ARG, "n_min must be >= 0");
  TuneRule* t = g_tune[fused_step];
  for (int r = 0; r < g_ntune[fused_step]; r++)
    if (t[r].n_min == n_min) {
      t[r].shape = shape;
      return GH_OK;
    }
  if (g_ntune[fused_step] >= kMaxTuneRules) return set_error(GH_ERR_ARG, "at most %d tuning rules", kMaxTuneRules);
  t[g_ntune[fused_step]++] = TuneRule{n_min, shape};
  return GH_OK;
}

int shape_for(int64_t n, int fused_step) {
  if (g_mixed_shape >= 0) return g_mixed_shape;
  return auto_shape(n, n, fused_step != 0);
}

int set_mixed_shape(int shape) {
  if (shape < 0) shape = -1;
  if (shape >= kNumMixedShapes) return set_error(GH_ERR_ARG, "mixed shape %d out of range", shape);
  g_mixed_shape = shape;
  return GH_OK;
}

// Mass-weighted centre of (pos, mass) into ws.origin[0..2], and the particles' common
// mass (0 when they differ) into ws.origin[3].
static int compute_origin(DirectWS& ws, const double* pos, const double* mass, int64_t n,
                          cudaStream_t st) {
  GH_TRY(ensure(ws.origin, 4 * sizeof(double)));
  GH_TRY(ensure(ws.com_part, COM_MAX_BLOCKS * (sizeof(dvec4) + sizeof(int))));
  int nb = (int)((n + 4 * COM_THREADS - 1) / (4 * COM_THREADS));
  if (nb < 1) nb = 1;
  if (nb > COM_MAX_BLOCKS) nb = COM_MAX_BLOCKS;
  dvec4* part = (dvec4*)ws.com_part.ptr;
  int* differ = (int*)(part + COM_MAX_BLOCKS);
  com_partial_kernel<<<nb, COM_THREADS, 0, st>>>(pos, mass, n, part, differ);
  GH_LAUNCH_CHECK();
  com_final_kernel<<<1, 32, 0, st>>>(part, differ, nb, mass, n, (double*)ws.origin.ptr);
  GH_LAUNCH_CHECK();
  return GH_OK;
}

static int ensure_streamk(DirectWS& ws, const StreamK& sk, int64_t slot_floats, cudaStream_t st) {
  GH_TRY(ensure(ws.partials, (size_t)(2 * sk.grid * slot_floats) * sizeof(float)));
  size_t cbytes = (size_t)sk.n_tiles * sizeof(int);
  if (ws.counters.bytes < cbytes || ws.counters_zeroed < cbytes) {
    GH_TRY(ensure(ws.counters, cbytes));
    GH_CUDA_TRY(cudaMemsetAsync(ws.counters.ptr, 0, ws.counters.bytes, st));
    ws.counters_zeroed = ws.counters.bytes;
  }
  return GH_OK;
}

template <class Epi>
static int launch_mixed(DirectWS& ws, const float4* src, int64_t np, const float4* tgt, int64_t nt,
                        double eps, const Epi& epi, cudaStream_t st) {
  DeviceInfo di;
  GH_TRY(device_info(&di));
  const float eps2 = (float)(eps * eps);
  const bool guard = !(eps2 > 0.f);
  const int shape = g_mixed_shape >= 0 ? g_mixed_shape : auto_shape(np, nt, Epi::kFusedStep);
  const MixedShape ms = kMixedShapes[shape];
  StreamK sk = mixed_plan(np, nt, mixed_grid_cap(di.num_sms, shape, guard), ms.threads * 2 * ms.packs,
                          ms.threads);
  if (sk.units == 0) return GH_OK;
  GH_TRY(ensure_streamk(ws, sk, mixed_slot_floats(ms.threads, ms.packs), st));
  float* partials = (float*)ws.partials.ptr;
  int* counters = (int*)ws.counters.ptr;
  prof_begin(st);
  // the sources' common mass, when they share one (compute_origin), else 0
  const double* eqm = (const double*)ws.origin.ptr + 3;
  if (guard)
    dispatch_shape<true>(shape, sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
  else
    dispatch_shape<false>(shape, sk, src, np, tgt, nt, eps2, partials, counters, epi, eqm, st);
  prof_end(st);
  GH_LAUNCH_CHECK();
  return GH_OK;
}

template <bool SELF, class Epi>
static int launch_f64(const double* spos, const double* smass, int64_t np, const double* tpos,
                      int64_t nt, double eps, const Epi& epi, cudaStream_t st) {
  const int64_t per = F64_THREADS * F64_R;
  const int64_t blocks = (nt + per - 1) / per;
  if (blocks == 0) return GH_OK;
  DeviceInfo di;
  GH_TRY(device_info(&di));
  const int64_t want = 2LL * di.num_sms;  // CTAs for a full machine
  int form = g_f64_form;
  // The thread-per-target kernel (90 registers, 5 CTAs per SM) fills the machine in
  // whole waves only from about 8 CTAs per SM; below that the CTA-wide kernel is
  // faster (N = 131,072: 447 against 562 ms; 262,144: 1780 against 1854 ms).
  if (form < 0) form = blocks < 8LL * di.num_sms ? 1 : 0;
  prof_begin(st);
  if (form == 0) {
    direct_f64_kernel<SELF, Epi><<<(unsigned)blocks, F64_THREADS, 0, st>>>(spos, smass, np, tpos, nt,
                                                                           eps * eps, epi);
  } else if ((nt + 7) / 8 >= want) {
    direct_f64_ordered_kernel<SELF, 8, Epi>
        <<<(unsigned)((nt + 7) / 8), F64O_THREADS, 0, st>>>(spos, smass, np, tpos, nt, eps * eps, epi);
  } else if ((nt + 3) / 4 >= want) {
    direct_f64_ordered_kernel<SELF, 4, Epi>
        <<<(unsigned)((nt + 3) / 4), F64O_THREADS, 0, st>>>(spos, smass, np, tpos, nt, eps * eps, epi);
  } else {
    direct_f64_ordered_kernel<SELF, 2, Epi>
        <<<(unsigned)((nt + 1) / 2), F64O_THREADS, 0, st>>>(spos, smass, np, tpos, nt, eps * eps, epi);
  }
  prof_end(st);
  GH_LAUNCH_CHECK();
  return GH_OK;
}

static int check_common(int64_t np, int64_t nt, double eps, int precision) {
  if (np < 0 || nt < 0) return set_error(GH_ERR_ARG, "negative particle count (np=%lld, nf=%lld)",
                                         (long long)np, (long long)nt);
  if (precision != GH_PREC_FP64 && precision != GH_PREC_MIXED)
    return set_error(GH_ERR_ARG, "unknown precision %d", precision);
  if (!(eps >= 0.0) || eps != eps) return set_error(GH_ERR_ARG, "eps must be >= 0 (got %g)", eps);
  return GH_OK;
}

int direct_force(const double* pos, const double* mass, int64_t np, const double* tpos, int64_t nt,
                 double eps, int precision, double* acc, cudaStream_t st) {
  GH_TRY(check_common(np, nt, eps, precision));
  const bool self = (tpos == nullptr);
  if (self) nt = np;
  if (nt == 0) return GH_OK;
  if (!acc || (np > 0 && (!pos || !mass)))
    return set_error(GH_ERR_ARG, "null buffer passed to direct force");
  if (np == 0) {
    GH_CUDA_TRY(cudaMemsetAsync(acc, 0, (size_t)nt * 3 * sizeof(double), st));
    return GH_OK;
  }
  EpiStore epi{acc};
  if (precision == GH_PREC_FP64) {
    if (self) return launch_f64<true>(pos, mass, np, pos, np, eps, epi, st);
    return launch_f64<false>(pos, mass, np, tpos, nt, eps, epi, st);
  }
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  DirectWS& ws = g_ws[di.device];
  GH_TRY(compute_origin(ws, pos, mass, np, st));
  GH_TRY(ensure(ws.src[0], (size_t)np * sizeof(float4)));
  const int T = 256;
  to_f32_kernel<<<(unsigned)((np + T - 1) / T), T, 0, st>>>(pos, mass, np, (const double*)ws.origin.ptr,
                                                           (float4*)ws.src[0].ptr);
  GH_LAUNCH_CHECK();
  const float4* tgt = (const float4*)ws.src[0].ptr;
  if (!self) {
    GH_TRY(ensure(ws.tgt, (size_t)nt * sizeof(float4)));
    to_f32_kernel<<<(unsigned)((nt + T - 1) / T), T, 0, st>>>(tpos, nullptr, nt,
                                                             (const double*)ws.origin.ptr,
                                                             (float4*)ws.tgt.ptr);
    GH_LAUNCH_CHECK();
    tgt = (const float4*)ws.tgt.ptr;
  }
  return launch_mixed(ws, (const float4*)ws.src[0].ptr, np, tgt, nt, eps, epi, st);
}

int drift_prepare_f64(const double* x, const double* v, int64_t n, double dt, double* xh, cudaStream_t st) {
  if (n == 0) return GH_OK;
  const int T = 256;
  drift_prepare_kernel<<<(unsigned)((n + T - 1) / T), T, 0, st>>>(x, v, nullptr, n, dt, nullptr, nullptr, xh);
  GH_LAUNCH_CHECK();
  return GH_OK;
}

int direct_run(double* x, double* v, const double* mass, int64_t np, int64_t nsteps, double dt,
               double eps, int precision, double* hist_x, double* hist_v, int64_t stride,
               cudaStream_t st) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  DirectWS& ws = g_ws[di.device];
  const int T = 256;
  const unsigned nb = (unsigned)((np + T - 1) / T);
  if (precision == GH_PREC_MIXED) {
    GH_TRY(compute_origin(ws, x, mass, np, st));
    GH_TRY(ensure(ws.src[0], (size_t)np * sizeof(float4)));
    GH_TRY(ensure(ws.src[1], (size_t)np * sizeof(float4)));
    drift_prepare_kernel<<<nb, T, 0, st>>>(x, v, mass, np, dt, (const double*)ws.origin.ptr,
                                           (float4*)ws.src[0].ptr, nullptr);
    GH_LAUNCH_CHECK();
  } else {
    GH_TRY(ensure(ws.xh[0], (size_t)np * 3 * sizeof(double)));
    GH_TRY(ensure(ws.xh[1], (size_t)np * 3 * sizeof(double)));
    drift_prepare_kernel<<<nb, T, 0, st>>>(x, v, mass, np, dt, nullptr, nullptr,
                                           (double*)ws.xh[0].ptr);
    GH_LAUNCH_CHECK();
  }
  for (int64_t s = 0; s < nsteps; s++) {
    Trace step("direct dkd step");
    const int cur = (int)(s & 1), nxt = cur ^ 1;
    EpiDKD epi;
    epi.x = x;
    epi.v = v;
    epi.mass = mass;
    epi.dt = dt;
    epi.hist_x = epi.hist_v = nullptr;
    if (hist_x && stride > 0 && (s + 1) % stride == 0) {
      const int64_t slot = (s + 1) / stride - 1;
      epi.hist_x = hist_x + slot * np * 3;
      epi.hist_v = hist_v + slot * np * 3;
    }
    if (precision == GH_PREC_MIXED) {
      epi.src_next = (float4*)ws.src[nxt].ptr;
      epi.xh_next = nullptr;
      epi.origin = (const double*)ws.origin.ptr;
      const float4* src = (const float4*)ws.src[cur].ptr;
      GH_TRY(launch_mixed(ws, src, np, src, np, eps, epi, st));
    } else {
      epi.src_next = nullptr;
      epi.xh_next = (double*)ws.xh[nxt].ptr;
      epi.origin = nullptr;
      const double* xh = (const double*)ws.xh[cur].ptr;
      GH_TRY(launch_f64<true>(xh, mass, np, xh, np, eps, epi, st));
    }
  }
  return GH_OK;
}

}  // namespace gh
