// Vector-Jacobian product of the direct-sum acceleration, and the softened
// potential, as all-pairs kernels.  Neither has a counterpart in the reference.
//
// With a_k = sum_j m_j d_kj / s_kj^{3/2}, d_kj = x_j - x_k, s_kj = |d_kj|^2 + eps^2, and
// an incoming cotangent lambda (N,3) on the code-unit accelerations:
//   dL/dx_k = sum_{j != k} [ q u - p (d.u) d ],   u = m_k lambda_j - m_j lambda_k,
//             q = s^{-3/2}, p = 3 s^{-5/2}   (the softened tidal tensor applied to u)
//   dL/dm_k = - sum_{j != k} q (lambda_j . d)
// Potential: phi_k = - sum_{j != k} m_j s^{-1/2}.
//
// Work split: a 2-D grid of (target tile, source split); each CTA writes per-target
// partial sums for its split to scratch and a reduction kernel adds the splits in
// split order, so results do not depend on scheduling.  FP64: one thread per target,
// s^{-1/2} from the hardware approximation refined by two Newton steps.  Mixed: FP32
// pair arithmetic on coordinates relative to the mass-weighted centre, per-chunk FP32
// partials folded into two-sum (hi, lo) accumulators, FP64 reduction.
#include <mutex>

#include "direct.cuh"
#include "engine.h"

namespace gh {

constexpr int AJ_THREADS = 128;

__device__ __forceinline__ double rsqrt_nr(double s) {
  double y;
  asm("rsqrt.approx.f64 %0, %1;" : "=d"(y) : "d"(s));
#pragma unroll
  for (int it = 0; it < 2; it++) {
    double e = fma(-s * y, y, 1.0);
    y = fma(0.5 * y, e, y);
  }
  return y;
}

// ---------------------------------------------------------------------------
// FP64 VJP: part[(split*n + k)*4 + {0,1,2,3}] = (gx, gy, gz, gm)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(AJ_THREADS)
    vjp_f64_kernel(const double* __restrict__ pos, const double* __restrict__ mass, const double* __restrict__ lam,
                   int64_t n, double eps2, int64_t jlen, double* __restrict__ part) {
  __shared__ dvec4 sp[AJ_THREADS], sl[AJ_THREADS];
  const int64_t k = (int64_t)blockIdx.x * AJ_THREADS + threadIdx.x;
  const int64_t split = blockIdx.y;
  const int64_t j0 = split * jlen, j1 = (j0 + jlen) < n ? j0 + jlen : n;
  const bool valid = k < n;
  const int64_t kk = valid ? k : 0;
  const double xk = pos[3 * kk], yk = pos[3 * kk + 1], zk = pos[3 * kk + 2], mk = mass[kk];
  const double lxk = lam[3 * kk], lyk = lam[3 * kk + 1], lzk = lam[3 * kk + 2];
  double gx = 0.0, gy = 0.0, gz = 0.0, gm = 0.0;
  for (int64_t c = j0; c < j1; c += AJ_THREADS) {
    __syncthreads();
    const int64_t j = c + threadIdx.x;
    if (j < j1) {
      sp[threadIdx.x] = make_dvec4(pos[3 * j], pos[3 * j + 1], pos[3 * j + 2], mass[j]);
      sl[threadIdx.x] = make_dvec4(lam[3 * j], lam[3 * j + 1], lam[3 * j + 2], 0.0);
    }
    __syncthreads();
    const int jn = (j1 - c) < AJ_THREADS ? (int)(j1 - c) : AJ_THREADS;
    for (int t = 0; t < jn; t++) {
      if (c + t == k) continue;
      const dvec4 P = sp[t], L = sl[t];
      const double dx = P.x - xk, dy = P.y - yk, dz = P.z - zk;
      const double s = fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2)));
      const double r = rsqrt_nr(s);
      const double r2 = r * r;
      const double q = r2 * r;
      const double p = 3.0 * q * r2;
      const double ux = mk * L.x - P.w * lxk, uy = mk * L.y - P.w * lyk, uz = mk * L.z - P.w * lzk;
      const double du = fma(dx, ux, fma(dy, uy, dz * uz));
      const double pd = p * du;
      gx = fma(q, ux, fma(-pd, dx, gx));
      gy = fma(q, uy, fma(-pd, dy, gy));
      gz = fma(q, uz, fma(-pd, dz, gz));
      gm = fma(-q, fma(L.x, dx, fma(L.y, dy, L.z * dz)), gm);
    }
  }
  if (valid) {
    double* o = part + (split * n + k) * 4;
    o[0] = gx;
    o[1] = gy;
    o[2] = gz;
    o[3] = gm;
  }
}

// ---------------------------------------------------------------------------
// Mixed VJP: FP32 pairs, 8 floats of partials per (split, target): hi/lo of gx..gm.
// ---------------------------------------------------------------------------
constexpr int AJ_CHUNK = AJ_THREADS;

__global__ void __launch_bounds__(AJ_THREADS)
    vjp_mixed_kernel(const float4* __restrict__ src, const float4* __restrict__ lsrc, int64_t n, float eps2,
                     int64_t jlen, float* __restrict__ part) {
  __shared__ float4 sp[AJ_CHUNK], sl[AJ_CHUNK];
  const int64_t k = (int64_t)blockIdx.x * AJ_THREADS + threadIdx.x;
  const int64_t split = blockIdx.y;
  const int64_t j0 = split * jlen, j1 = (j0 + jlen) < n ? j0 + jlen : n;
  const bool valid = k < n;
  const float4 T = valid ? src[k] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 TL = valid ? lsrc[k] : make_float4(0.f, 0.f, 0.f, 0.f);
  float h[4] = {0.f, 0.f, 0.f, 0.f}, l[4] = {0.f, 0.f, 0.f, 0.f};
  for (int64_t c = j0; c < j1; c += AJ_CHUNK) {
    __syncthreads();
    const int64_t j = c + threadIdx.x;
    // padding and the target itself contribute nothing: zero mass and zero lambda
    sp[threadIdx.x] = j < j1 ? src[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    sl[threadIdx.x] = j < j1 ? lsrc[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    float gx = 0.f, gy = 0.f, gz = 0.f, gm = 0.f;
#pragma unroll 4
    for (int t = 0; t < AJ_CHUNK; t++) {
      const float4 P = sp[t], L = sl[t];
      const float dx = P.x - T.x, dy = P.y - T.y, dz = P.z - T.z;
      const float s = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
      float r = rsqrt_approx(s);
      r = (c + t == k || !(s > 0.f)) ? 0.f : r;
      const float r2 = r * r;
      const float q = r2 * r;
      const float p = 3.f * q * r2;
      const float ux = fmaf(T.w, L.x, -P.w * TL.x), uy = fmaf(T.w, L.y, -P.w * TL.y),
                  uz = fmaf(T.w, L.z, -P.w * TL.z);
      const float pd = p * fmaf(dx, ux, fmaf(dy, uy, dz * uz));
      gx = fmaf(q, ux, fmaf(-pd, dx, gx));
      gy = fmaf(q, uy, fmaf(-pd, dy, gy));
      gz = fmaf(q, uz, fmaf(-pd, dz, gz));
      gm = fmaf(-q, fmaf(L.x, dx, fmaf(L.y, dy, L.z * dz)), gm);
    }
    const float pv[4] = {gx, gy, gz, gm};
#pragma unroll
    for (int q = 0; q < 4; q++) {
      float s, e;
      two_sum(h[q], pv[q], s, e);
      h[q] = s;
      l[q] = __fadd_rn(l[q], e);
    }
  }
  if (valid) {
    float* o = part + (split * n + k) * 8;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      o[2 * q] = h[q];
      o[2 * q + 1] = l[q];
    }
  }
}

__global__ void vjp_reduce_f64_kernel(const double* __restrict__ part, int splits, int64_t n,
                                      double* __restrict__ gpos, double* __restrict__ gmass) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double a[4] = {0.0, 0.0, 0.0, 0.0};
  for (int s = 0; s < splits; s++)
    for (int q = 0; q < 4; q++) a[q] += part[((int64_t)s * n + k) * 4 + q];
  gpos[3 * k] = a[0];
  gpos[3 * k + 1] = a[1];
  gpos[3 * k + 2] = a[2];
  if (gmass) gmass[k] = a[3];
}

__global__ void vjp_reduce_mixed_kernel(const float* __restrict__ part, int splits, int64_t n,
                                        double* __restrict__ gpos, double* __restrict__ gmass) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double a[4] = {0.0, 0.0, 0.0, 0.0};
  for (int s = 0; s < splits; s++)
    for (int q = 0; q < 4; q++) {
      const float* o = part + ((int64_t)s * n + k) * 8;
      a[q] += (double)o[2 * q] + (double)o[2 * q + 1];
    }
  gpos[3 * k] = a[0];
  gpos[3 * k + 1] = a[1];
  gpos[3 * k + 2] = a[2];
  if (gmass) gmass[k] = a[3];
}

// ---------------------------------------------------------------------------
// Potential, FP64: part[split*n + k] = -sum_{j in split, j != k} m_j s^{-1/2}
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(AJ_THREADS)
    potential_f64_kernel(const double* __restrict__ pos, const double* __restrict__ mass, int64_t n, double eps2,
                         int64_t jlen, double* __restrict__ part) {
  __shared__ dvec4 sp[AJ_THREADS];
  const int64_t k = (int64_t)blockIdx.x * AJ_THREADS + threadIdx.x;
  const int64_t split = blockIdx.y;
  const int64_t j0 = split * jlen, j1 = (j0 + jlen) < n ? j0 + jlen : n;
  const bool valid = k < n;
  const int64_t kk = valid ? k : 0;
  const double xk = pos[3 * kk], yk = pos[3 * kk + 1], zk = pos[3 * kk + 2];
  double phi = 0.0;
  for (int64_t c = j0; c < j1; c += AJ_THREADS) {
    __syncthreads();
    const int64_t j = c + threadIdx.x;
    if (j < j1) sp[threadIdx.x] = make_dvec4(pos[3 * j], pos[3 * j + 1], pos[3 * j + 2], mass[j]);
    __syncthreads();
    const int jn = (j1 - c) < AJ_THREADS ? (int)(j1 - c) : AJ_THREADS;
    for (int t = 0; t < jn; t++) {
      if (c + t == k) continue;
      const dvec4 P = sp[t];
      const double dx = P.x - xk, dy = P.y - yk, dz = P.z - zk;
      const double s = fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2)));
      if (s > 0.0) phi = fma(-P.w, rsqrt_nr(s), phi);
    }
  }
  if (valid) part[split * n + k] = phi;
}

__global__ void potential_reduce_kernel(const double* __restrict__ part, int splits, int64_t n,
                                        double* __restrict__ phi) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double a = 0.0;
  for (int s = 0; s < splits; s++) a += part[(int64_t)s * n + k];
  phi[k] = a;
}

// FP32 relative sources (x, y, z, m) and cotangents (lx, ly, lz, 0).
__global__ void vjp_prepare_mixed_kernel(const double* __restrict__ pos, const double* __restrict__ mass,
                                         const double* __restrict__ lam, int64_t n, const double* __restrict__ origin,
                                         float4* __restrict__ src, float4* __restrict__ lsrc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  src[i] = make_float4((float)(pos[3 * i] - origin[0]), (float)(pos[3 * i + 1] - origin[1]),
                       (float)(pos[3 * i + 2] - origin[2]), (float)mass[i]);
  lsrc[i] = make_float4((float)lam[3 * i], (float)lam[3 * i + 1], (float)lam[3 * i + 2], 0.f);
}

__global__ void mean_origin_kernel(const double* __restrict__ pos, const double* __restrict__ mass, int64_t n,
                                   double* __restrict__ origin) {
  __shared__ dvec4 red[256];
  dvec4 a = make_dvec4(0.0, 0.0, 0.0, 0.0);
  for (int64_t i = threadIdx.x; i < n; i += 256) {
    const double m = mass[i];
    a.x += m * pos[3 * i];
    a.y += m * pos[3 * i + 1];
    a.z += m * pos[3 * i + 2];
    a.w += m;
  }
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
    origin[0] = ok ? r.x / r.w : 0.0;
    origin[1] = ok ? r.y / r.w : 0.0;
    origin[2] = ok ? r.z / r.w : 0.0;
  }
}

// ---------------------------------------------------------------------------
struct AdjWS {
  Buffer part, src, lsrc, origin;
};
static AdjWS g_adj[64];
static std::mutex g_adj_mu;

// Number of source splits so that the grid fills the GPU about twice over.
static int64_t choose_splits(int64_t n, int num_sms) {
  const int64_t tiles = (n + AJ_THREADS - 1) / AJ_THREADS;
  int64_t want = (4LL * num_sms * 4 + tiles - 1) / tiles;  // ~4 CTAs of 128 threads per SM, x4
  const int64_t max_splits = (n + AJ_THREADS - 1) / AJ_THREADS;
  if (want > max_splits) want = max_splits;
  if (want < 1) want = 1;
  return want;
}

int direct_vjp(const double* pos, const double* mass, int64_t n, double eps, const double* lam, int precision,
               double* gpos, double* gmass, cudaStream_t st) {
  if (n < 0) return set_error(GH_ERR_ARG, "negative particle count");
  if (!(eps >= 0.0)) return set_error(GH_ERR_ARG, "eps must be >= 0 (got %g)", eps);
  if (precision != GH_PREC_FP64 && precision != GH_PREC_MIXED)
    return set_error(GH_ERR_ARG, "unknown precision %d", precision);
  if (n == 0) return GH_OK;
  if (!pos || !mass || !lam || !gpos) return set_error(GH_ERR_ARG, "null buffer");
  std::lock_guard<std::mutex> lk(g_adj_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  AdjWS& ws = g_adj[di.device];
  const int64_t splits = choose_splits(n, di.num_sms);
  const int64_t jlen = (n + splits - 1) / splits;
  const dim3 grid((unsigned)((n + AJ_THREADS - 1) / AJ_THREADS), (unsigned)splits);
  const unsigned rb = (unsigned)((n + 255) / 256);
  if (precision == GH_PREC_FP64) {
    GH_TRY(ensure(ws.part, (size_t)splits * n * 4 * sizeof(double)));
    prof_begin(st);
    vjp_f64_kernel<<<grid, AJ_THREADS, 0, st>>>(pos, mass, lam, n, eps * eps, jlen, (double*)ws.part.ptr);
    prof_end(st);
    GH_LAUNCH_CHECK();
    vjp_reduce_f64_kernel<<<rb, 256, 0, st>>>((const double*)ws.part.ptr, (int)splits, n, gpos, gmass);
    GH_LAUNCH_CHECK();
    return GH_OK;
  }
  GH_TRY(ensure(ws.part, (size_t)splits * n * 8 * sizeof(float)));
  GH_TRY(ensure(ws.src, (size_t)n * sizeof(float4)));
  GH_TRY(ensure(ws.lsrc, (size_t)n * sizeof(float4)));
  GH_TRY(ensure(ws.origin, 4 * sizeof(double)));
  mean_origin_kernel<<<1, 256, 0, st>>>(pos, mass, n, (double*)ws.origin.ptr);
  GH_LAUNCH_CHECK();
  vjp_prepare_mixed_kernel<<<rb, 256, 0, st>>>(pos, mass, lam, n, (const double*)ws.origin.ptr, (float4*)ws.src.ptr,
                                               (float4*)ws.lsrc.ptr);
  GH_LAUNCH_CHECK();
  prof_begin(st);
  vjp_mixed_kernel<<<grid, AJ_THREADS, 0, st>>>((const float4*)ws.src.ptr, (const float4*)ws.lsrc.ptr, n,
                                                (float)(eps * eps), jlen, (float*)ws.part.ptr);
  prof_end(st);
  GH_LAUNCH_CHECK();
  vjp_reduce_mixed_kernel<<<rb, 256, 0, st>>>((const float*)ws.part.ptr, (int)splits, n, gpos, gmass);
  GH_LAUNCH_CHECK();
  return GH_OK;
}

int potential(const double* pos, const double* mass, int64_t n, double eps, double* phi, cudaStream_t st) {
  if (n < 0) return set_error(GH_ERR_ARG, "negative particle count");
  if (!(eps >= 0.0)) return set_error(GH_ERR_ARG, "eps must be >= 0 (got %g)", eps);
  if (n == 0) return GH_OK;
  if (!pos || !mass || !phi) return set_error(GH_ERR_ARG, "null buffer");
  std::lock_guard<std::mutex> lk(g_adj_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  AdjWS& ws = g_adj[di.device];
  const int64_t splits = choose_splits(n, di.num_sms);
  const int64_t jlen = (n + splits - 1) / splits;
  GH_TRY(ensure(ws.part, (size_t)splits * n * sizeof(double)));
  const dim3 grid((unsigned)((n + AJ_THREADS - 1) / AJ_THREADS), (unsigned)splits);
  potential_f64_kernel<<<grid, AJ_THREADS, 0, st>>>(pos, mass, n, eps * eps, jlen, (double*)ws.part.ptr);
  GH_LAUNCH_CHECK();
  potential_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const double*)ws.part.ptr, (int)splits, n,
                                                                       phi);
  GH_LAUNCH_CHECK();
  return GH_OK;
}

}  // namespace gh
