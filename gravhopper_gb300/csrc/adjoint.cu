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
      double r2, q;  // s^-1 and s^(-3/2) on the integer pipes; FP64 Newton steps outside its range
      if (!emu::rsqrt_powers(s, r2, q)) {
        const double r = rsqrt_nr(s);
        r2 = r * r;
        q = r2 * r;
      }
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
// Mixed VJP: FP32 pair arithmetic on packed f32x2 lanes (two targets per thread
// register pair, VJ_P packs per thread), sources duplicated per lane pair in shared
// memory, per-chunk partials folded into two-sum (hi, lo) accumulators; 8 floats of
// partials per (split, target): hi/lo of gx, gy, gz, gm.  Per pair: 30 FP32 lane-ops
// (3 sub, 3 fma for s, 4 for q and -3q/s, 6 for u (3 with equal masses), 3 for d.u,
// 1, 6 for g, 4 for gm) and one MUFU rsqrt.
// ---------------------------------------------------------------------------
constexpr int VJ_THREADS = 128;
constexpr int VJ_P = 2;
constexpr int VJ_TILE = VJ_THREADS * 2 * VJ_P;
constexpr int VJ_JT = VJ_THREADS;

// EQ (all masses equal): u = m (lambda_j - lambda_k) with the mass taken out, one
// subtraction instead of a product and an FMA per component; the caller scales the
// position gradient by m once (the mass gradient's terms hold no mass).
template <bool SELFCHK, bool EQ = false>
__device__ __forceinline__ void vjp_chunk(const float4* __restrict__ tile, int64_t jbase, const int64_t* ka,
                                          const f2* tx, const f2* ty, const f2* tz, const f2* tm, const f2* tlx,
                                          const f2* tly, const f2* tlz, f2 E2, f2* gx, f2* gy, f2* gz, f2* gm) {
  const f2 M3 = f2make(-3.f, -3.f);
#pragma unroll 2
  for (int k = 0; k < VJ_JT; k++) {
    const float4 A = tile[4 * k], B = tile[4 * k + 1], C = tile[4 * k + 2], D = tile[4 * k + 3];
    const f2 X = f2make(A.x, A.y), Y = f2make(A.z, A.w), Z = f2make(B.x, B.y), NM = f2make(B.z, B.w);
    const f2 LX = f2make(C.x, C.y), LY = f2make(C.z, C.w), LZ = f2make(D.x, D.y);
#pragma unroll
    for (int p = 0; p < VJ_P; p++) {
      const f2 dx = f2sub(X, tx[p]), dy = f2sub(Y, ty[p]), dz = f2sub(Z, tz[p]);
      f2 s = f2fma(dx, dx, E2);
      s = f2fma(dy, dy, s);
      s = f2fma(dz, dz, s);
      float sa, sb;
      f2split(s, sa, sb);
      float ra = rsqrt_approx(sa), rb = rsqrt_approx(sb);
      if (SELFCHK) {
        ra = (jbase + k == ka[2 * p]) ? 0.f : ra;
        rb = (jbase + k == ka[2 * p + 1]) ? 0.f : rb;
      }
      const f2 r = f2make(ra, rb);
      const f2 r2 = f2mul(r, r);
      const f2 q = f2mul(r2, r);
      const f2 np = f2mul(f2mul(q, M3), r2);
      const f2 ux = EQ ? f2sub(LX, tlx[p]) : f2fma(NM, tlx[p], f2mul(tm[p], LX));
      const f2 uy = EQ ? f2sub(LY, tly[p]) : f2fma(NM, tly[p], f2mul(tm[p], LY));
      const f2 uz = EQ ? f2sub(LZ, tlz[p]) : f2fma(NM, tlz[p], f2mul(tm[p], LZ));
      f2 du = f2mul(dx, ux);
      du = f2fma(dy, uy, du);
      du = f2fma(dz, uz, du);
      const f2 npd = f2mul(np, du);
      gx[p] = f2fma(npd, dx, f2fma(q, ux, gx[p]));
      gy[p] = f2fma(npd, dy, f2fma(q, uy, gy[p]));
      gz[p] = f2fma(npd, dz, f2fma(q, uz, gz[p]));
      f2 ld = f2mul(dx, LX);
      ld = f2fma(dy, LY, ld);
      ld = f2fma(dz, LZ, ld);
      gm[p] = f2fma(q, ld, gm[p]);
    }
  }
}

__global__ void __launch_bounds__(VJ_THREADS, 4)
    vjp_mixed_kernel(const float4* __restrict__ src, const float4* __restrict__ lsrc, int64_t n, float eps2,
                     int64_t jlen, float* __restrict__ part, const double* __restrict__ meqp) {
  __shared__ __align__(16) float4 tile[4 * VJ_JT];
  const int tid = threadIdx.x;
  const int64_t tbase = (int64_t)blockIdx.x * VJ_TILE;
  const int64_t split = blockIdx.y;
  const int64_t j0 = split * jlen, j1 = (j0 + jlen) < n ? j0 + jlen : n;
  // equal masses: the sums are taken with unit masses (staged as such for the general
  // loop of a partial chunk: -1 for a source, 0 for padding, 1 for every target) and the
  // position gradient is scaled by the mass in the reduction
  const bool eq = __ldg(meqp) != 0.0;
  f2 tx[VJ_P], ty[VJ_P], tz[VJ_P], tm[VJ_P], tlx[VJ_P], tly[VJ_P], tlz[VJ_P];
  f2 hx[VJ_P], hy[VJ_P], hz[VJ_P], hm[VJ_P], lx[VJ_P], ly[VJ_P], lz[VJ_P], lm[VJ_P];
  int64_t ka[2 * VJ_P];
#pragma unroll
  for (int p = 0; p < VJ_P; p++) {
    float4 P0[2], L0[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int64_t k = tbase + (2 * p + h) * VJ_THREADS + tid;
      ka[2 * p + h] = k;
      P0[h] = k < n ? src[k] : make_float4(0.f, 0.f, 0.f, 0.f);
      L0[h] = k < n ? lsrc[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    tx[p] = f2make(P0[0].x, P0[1].x);
    ty[p] = f2make(P0[0].y, P0[1].y);
    tz[p] = f2make(P0[0].z, P0[1].z);
    tm[p] = eq ? f2make(1.f, 1.f) : f2make(P0[0].w, P0[1].w);
    tlx[p] = f2make(L0[0].x, L0[1].x);
    tly[p] = f2make(L0[0].y, L0[1].y);
    tlz[p] = f2make(L0[0].z, L0[1].z);
    hx[p] = hy[p] = hz[p] = hm[p] = lx[p] = ly[p] = lz[p] = lm[p] = 0ull;
  }
  const f2 E2 = f2make(eps2, eps2);
  for (int64_t c = j0; c < j1; c += VJ_JT) {
    __syncthreads();
    {
      const int64_t j = c + tid;
      const float4 P = j < j1 ? src[j] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 L = j < j1 ? lsrc[j] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float w = eq ? (j < j1 ? 1.f : 0.f) : P.w;
      tile[4 * tid + 0] = make_float4(P.x, P.x, P.y, P.y);
      tile[4 * tid + 1] = make_float4(P.z, P.z, -w, -w);
      tile[4 * tid + 2] = make_float4(L.x, L.x, L.y, L.y);
      tile[4 * tid + 3] = make_float4(L.z, L.z, 0.f, 0.f);
    }
    __syncthreads();
    f2 gx[VJ_P], gy[VJ_P], gz[VJ_P], gm[VJ_P];
#pragma unroll
    for (int p = 0; p < VJ_P; p++) gx[p] = gy[p] = gz[p] = gm[p] = 0ull;
    // only a chunk that overlaps this tile's targets can pair a target with itself
    const bool self = c < tbase + VJ_TILE && c + VJ_JT > tbase;
    if (eq && c + VJ_JT <= j1) {  // a full chunk of equal masses
      if (self)
        vjp_chunk<true, true>(tile, c, ka, tx, ty, tz, tm, tlx, tly, tlz, E2, gx, gy, gz, gm);
      else
        vjp_chunk<false, true>(tile, c, ka, tx, ty, tz, tm, tlx, tly, tlz, E2, gx, gy, gz, gm);
    } else {
      if (self)
        vjp_chunk<true>(tile, c, ka, tx, ty, tz, tm, tlx, tly, tlz, E2, gx, gy, gz, gm);
      else
        vjp_chunk<false>(tile, c, ka, tx, ty, tz, tm, tlx, tly, tlz, E2, gx, gy, gz, gm);
    }
#pragma unroll
    for (int p = 0; p < VJ_P; p++) {
      f2 sm, e;
      f2two_sum(hx[p], gx[p], sm, e);
      hx[p] = sm;
      lx[p] = f2add(lx[p], e);
      f2two_sum(hy[p], gy[p], sm, e);
      hy[p] = sm;
      ly[p] = f2add(ly[p], e);
      f2two_sum(hz[p], gz[p], sm, e);
      hz[p] = sm;
      lz[p] = f2add(lz[p], e);
      f2two_sum(hm[p], gm[p], sm, e);
      hm[p] = sm;
      lm[p] = f2add(lm[p], e);
    }
  }
#pragma unroll
  for (int p = 0; p < VJ_P; p++) {
    float a[8], b[8];
    f2split(hx[p], a[0], b[0]);
    f2split(lx[p], a[1], b[1]);
    f2split(hy[p], a[2], b[2]);
    f2split(ly[p], a[3], b[3]);
    f2split(hz[p], a[4], b[4]);
    f2split(lz[p], a[5], b[5]);
    f2split(hm[p], a[6], b[6]);
    f2split(lm[p], a[7], b[7]);
    // dL/dm_k = -sum q (lambda_j . d): the mass terms were accumulated with + sign
    a[6] = -a[6];
    a[7] = -a[7];
    b[6] = -b[6];
    b[7] = -b[7];
    const int64_t k0 = ka[2 * p], k1 = ka[2 * p + 1];
    if (k0 < n) {
      float* o = part + (split * n + k0) * 8;
#pragma unroll
      for (int q = 0; q < 8; q++) o[q] = a[q];
    }
    if (k1 < n) {
      float* o = part + (split * n + k1) * 8;
#pragma unroll
      for (int q = 0; q < 8; q++) o[q] = b[q];
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
                                        const double* __restrict__ meqp, double* __restrict__ gpos,
                                        double* __restrict__ gmass) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double a[4] = {0.0, 0.0, 0.0, 0.0};
  for (int s = 0; s < splits; s++)
    for (int q = 0; q < 4; q++) {
      const float* o = part + ((int64_t)s * n + k) * 8;
      a[q] += (double)o[2 * q] + (double)o[2 * q + 1];
    }
  const double meq = *meqp;
  const double sm = meq != 0.0 ? meq : 1.0;  // equal masses: the sums were taken with unit masses
  gpos[3 * k] = sm * a[0];
  gpos[3 * k + 1] = sm * a[1];
  gpos[3 * k + 2] = sm * a[2];
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
      if (s > 0.0) {
        double y;  // s^(-1/2) on the integer pipes; FP64 Newton steps outside its range
        if (!emu::rsqrt1(s, y)) y = rsqrt_nr(s);
        phi = fma(-P.w, y, phi);
      }
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

// origin[0..2]: the mass-weighted centre; origin[3]: the common mass when every mass
// equals the first (finite, nonzero; a NaN never does), else 0.
__global__ void mean_origin_kernel(const double* __restrict__ pos, const double* __restrict__ mass, int64_t n,
                                   double* __restrict__ origin) {
  __shared__ dvec4 red[256];
  const double m0 = n > 0 ? mass[0] : 0.0;
  dvec4 a = make_dvec4(0.0, 0.0, 0.0, 0.0);
  bool ne = false;
  for (int64_t i = threadIdx.x; i < n; i += 256) {
    const double m = mass[i];
    ne |= !(m == m0);
    a.x += m * pos[3 * i];
    a.y += m * pos[3 * i + 1];
    a.z += m * pos[3 * i + 2];
    a.w += m;
  }
  ne = __syncthreads_or(ne);
  if (threadIdx.x == 0) origin[3] = (!ne && m0 != 0.0 && isfinite(m0)) ? m0 : 0.0;
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
  GH_TRY(ensure(ws.src, (size_t)n * sizeof(float4)));
  GH_TRY(ensure(ws.lsrc, (size_t)n * sizeof(float4)));
  GH_TRY(ensure(ws.origin, 4 * sizeof(double)));
  mean_origin_kernel<<<1, 256, 0, st>>>(pos, mass, n, (double*)ws.origin.ptr);
  GH_LAUNCH_CHECK();
  vjp_prepare_mixed_kernel<<<rb, 256, 0, st>>>(pos, mass, lam, n, (const double*)ws.origin.ptr, (float4*)ws.src.ptr,
                                               (float4*)ws.lsrc.ptr);
  GH_LAUNCH_CHECK();
  // Mixed kernel: tiles of VJ_TILE targets, splits of whole VJ_JT-source chunks,
  // about four resident CTAs per SM, filled twice over.
  const int64_t mtiles = (n + VJ_TILE - 1) / VJ_TILE;
  const int64_t chunks = (n + VJ_JT - 1) / VJ_JT;
  int64_t msplits = (8LL * di.num_sms + mtiles - 1) / mtiles;
  if (msplits > chunks) msplits = chunks;
  if (msplits < 1) msplits = 1;
  const int64_t mjlen = ((chunks + msplits - 1) / msplits) * VJ_JT;
  msplits = (n + mjlen - 1) / mjlen;
  GH_TRY(ensure(ws.part, (size_t)msplits * n * 8 * sizeof(float)));
  prof_begin(st);
  vjp_mixed_kernel<<<dim3((unsigned)mtiles, (unsigned)msplits), VJ_THREADS, 0, st>>>(
      (const float4*)ws.src.ptr, (const float4*)ws.lsrc.ptr, n, (float)(eps * eps), mjlen, (float*)ws.part.ptr,
      (const double*)ws.origin.ptr + 3);
  prof_end(st);
  GH_LAUNCH_CHECK();
  vjp_reduce_mixed_kernel<<<rb, 256, 0, st>>>((const float*)ws.part.ptr, (int)msplits, n,
                                              (const double*)ws.origin.ptr + 3, gpos, gmass);
  GH_LAUNCH_CHECK();
  return GH_OK;
}

// ---------------------------------------------------------------------------
// Backward pass of drift-kick-drift steps.  Forward step (gravhopper.py:405-416):
//   xh = x + c v,  v' = v + dt A F(xh),  x' = xh + c v'      (c = 0.5 dt F_kpc)
// Reverse, given (xbar, vbar) of (x', v'):
//   w = vbar + c xbar;  lam = A dt w;  (gx, gm) = VJP of F at xh with lam;
//   xhbar = xbar + gx;  xbar <- xhbar;  vbar <- w + c xhbar;  mbar += gm
// ---------------------------------------------------------------------------
__global__ void adj_pre_kernel(const double* __restrict__ x, const double* __restrict__ v, int64_t n, double dt,
                               const double* __restrict__ xbar, const double* __restrict__ vbar,
                               double* __restrict__ xh, double* __restrict__ w, double* __restrict__ lam) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * n) return;
  const double c = 0.5 * dt * GH_KMS_MYR_TO_KPC;
  xh[i] = drift_half(x[i], v[i], dt);
  const double wi = vbar[i] + c * xbar[i];
  w[i] = wi;
  lam[i] = (GH_ACCEL_UNIT * dt) * wi;
}

__global__ void adj_post_kernel(int64_t n, double dt, const double* __restrict__ w, const double* __restrict__ gpos,
                                const double* __restrict__ gmass, double* __restrict__ xbar,
                                double* __restrict__ vbar, double* __restrict__ mbar) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 3 * n) {
    const double c = 0.5 * dt * GH_KMS_MYR_TO_KPC;
    const double xhb = xbar[i] + gpos[i];
    xbar[i] = xhb;
    vbar[i] = w[i] + c * xhb;
  }
  if (i < n && mbar) mbar[i] += gmass[i];
}

struct BwdWS {
  Buffer states_x, states_v, work_x, work_v, xh, w, lam, gpos, gmass;
  Buffer chain_x[2], chain_v[2];        // dkd_backward_chain: recomputed segments, two buffers
  cudaStream_t rstream = nullptr;       // dkd_backward_chain: recomputation stream
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
};
static BwdWS g_bwd[64];
static std::mutex g_bwd_mu;

// Back-propagates through `nsteps` recomputed states (sx, sv: state at the start of
// each step) with the VJP kernel: (xbar, vbar) updated in place, mbar incremented.
static int backward_steps(BwdWS& ws, const double* sx, const double* sv, const double* mass, int64_t n,
                          int64_t nsteps, double dt, double eps, int precision, double* xbar, double* vbar,
                          double* mbar, cudaStream_t st) {
  const unsigned b3 = (unsigned)((3 * n + 255) / 256);
  for (int64_t j = nsteps - 1; j >= 0; j--) {
    adj_pre_kernel<<<b3, 256, 0, st>>>(sx + 3 * n * j, sv + 3 * n * j, n, dt, xbar, vbar, (double*)ws.xh.ptr,
                                       (double*)ws.w.ptr, (double*)ws.lam.ptr);
    GH_LAUNCH_CHECK();
    GH_TRY(direct_vjp((const double*)ws.xh.ptr, mass, n, eps, (const double*)ws.lam.ptr, precision,
                      (double*)ws.gpos.ptr, (double*)ws.gmass.ptr, st));
    adj_post_kernel<<<b3, 256, 0, st>>>(n, dt, (const double*)ws.w.ptr, (const double*)ws.gpos.ptr,
                                        (const double*)ws.gmass.ptr, xbar, vbar, mbar);
    GH_LAUNCH_CHECK();
  }
  return GH_OK;
}

int dkd_backward(const double* x0, const double* v0, const double* mass, int64_t n, int64_t nsteps, double dt,
                 double eps, int precision, double* xbar, double* vbar, double* mbar, cudaStream_t st) {
  if (n < 0 || nsteps < 0) return set_error(GH_ERR_ARG, "negative n or nsteps");
  if (n == 0 || nsteps == 0) return GH_OK;
  if (!x0 || !v0 || !mass || !xbar || !vbar) return set_error(GH_ERR_ARG, "null buffer");
  std::lock_guard<std::mutex> lk(g_bwd_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  BwdWS& ws = g_bwd[di.device];
  const size_t vec = (size_t)n * 3 * sizeof(double);
  GH_TRY(ensure(ws.states_x, vec * nsteps));
  GH_TRY(ensure(ws.states_v, vec * nsteps));
  GH_TRY(ensure(ws.work_x, vec));
  GH_TRY(ensure(ws.work_v, vec));
  GH_TRY(ensure(ws.xh, vec));
  GH_TRY(ensure(ws.w, vec));
  GH_TRY(ensure(ws.lam, vec));
  GH_TRY(ensure(ws.gpos, vec));
  GH_TRY(ensure(ws.gmass, (size_t)n * sizeof(double)));
  double* sx = (double*)ws.states_x.ptr;
  double* sv = (double*)ws.states_v.ptr;
  // states[j] = state at the start of step j, j = 0 .. nsteps-1, recomputed from x0, v0
  GH_CUDA_TRY(cudaMemcpyAsync(sx, x0, vec, cudaMemcpyDeviceToDevice, st));
  GH_CUDA_TRY(cudaMemcpyAsync(sv, v0, vec, cudaMemcpyDeviceToDevice, st));
  if (nsteps > 1) {
    GH_CUDA_TRY(cudaMemcpyAsync(ws.work_x.ptr, x0, vec, cudaMemcpyDeviceToDevice, st));
    GH_CUDA_TRY(cudaMemcpyAsync(ws.work_v.ptr, v0, vec, cudaMemcpyDeviceToDevice, st));
    GH_TRY(direct_run((double*)ws.work_x.ptr, (double*)ws.work_v.ptr, mass, n, nsteps - 1, dt, eps, precision,
                      sx + 3 * n, sv + 3 * n, 1, st));
  }
  return backward_steps(ws, sx, sv, mass, n, nsteps, dt, eps, precision, xbar, vbar, mbar, st);
}

// Multi-segment form: the checkpoints of all segments at once; segment s-1 is
// recomputed on a second stream while segment s back-propagates on `st` (two state
// buffers, ordered by events), so the recomputation overlaps the VJP launches.
int dkd_backward_chain(const double* cx, const double* cv, const int64_t* seg, int64_t nseg, const double* mass,
                       int64_t n, double dt, double eps, int precision, double* xbar, double* vbar, double* mbar,
                       cudaStream_t st) {
  if (n < 0 || nseg < 0) return set_error(GH_ERR_ARG, "negative n or segment count");
  if (n == 0 || nseg == 0) return GH_OK;
  if (!cx || !cv || !seg || !mass || !xbar || !vbar) return set_error(GH_ERR_ARG, "null buffer");
  int64_t maxseg = 0;
  for (int64_t s = 0; s < nseg; s++) {
    if (seg[s] < 1) return set_error(GH_ERR_ARG, "segment %lld has %lld steps", (long long)s, (long long)seg[s]);
    if (seg[s] > maxseg) maxseg = seg[s];
  }
  std::lock_guard<std::mutex> lk(g_bwd_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  BwdWS& ws = g_bwd[di.device];
  const size_t vec = (size_t)n * 3 * sizeof(double);
  for (int b = 0; b < 2; b++) {
    GH_TRY(ensure(ws.chain_x[b], vec * maxseg));
    GH_TRY(ensure(ws.chain_v[b], vec * maxseg));
  }
  GH_TRY(ensure(ws.work_x, vec));
  GH_TRY(ensure(ws.work_v, vec));
  GH_TRY(ensure(ws.xh, vec));
  GH_TRY(ensure(ws.w, vec));
  GH_TRY(ensure(ws.lam, vec));
  GH_TRY(ensure(ws.gpos, vec));
  GH_TRY(ensure(ws.gmass, (size_t)n * sizeof(double)));
  if (!ws.rstream) {
    GH_CUDA_TRY(cudaStreamCreateWithFlags(&ws.rstream, cudaStreamNonBlocking));
    for (int b = 0; b < 3; b++) GH_CUDA_TRY(cudaEventCreateWithFlags(&ws.ev[b], cudaEventDisableTiming));
  }
  cudaStream_t rs = ws.rstream;
  cudaEvent_t ev_ready[2] = {ws.ev[0], ws.ev[1]};  // recomputed segment in buffer b
  cudaEvent_t ev_free = ws.ev[2];                  // the backward that last read a buffer
  GH_CUDA_TRY(cudaEventRecord(ev_free, st));        // the caller's work before anything here
  GH_CUDA_TRY(cudaStreamWaitEvent(rs, ev_free, 0));
  auto recompute = [&](int64_t s) -> int {
    const int b = (int)(s & 1);
    double* sx = (double*)ws.chain_x[b].ptr;
    double* sv = (double*)ws.chain_v[b].ptr;
    GH_CUDA_TRY(cudaMemcpyAsync(sx, cx + 3 * n * s, vec, cudaMemcpyDeviceToDevice, rs));
    GH_CUDA_TRY(cudaMemcpyAsync(sv, cv + 3 * n * s, vec, cudaMemcpyDeviceToDevice, rs));
    if (seg[s] > 1) {
      GH_CUDA_TRY(cudaMemcpyAsync(ws.work_x.ptr, cx + 3 * n * s, vec, cudaMemcpyDeviceToDevice, rs));
      GH_CUDA_TRY(cudaMemcpyAsync(ws.work_v.ptr, cv + 3 * n * s, vec, cudaMemcpyDeviceToDevice, rs));
      GH_TRY(direct_run((double*)ws.work_x.ptr, (double*)ws.work_v.ptr, mass, n, seg[s] - 1, dt, eps, precision,
                        sx + 3 * n, sv + 3 * n, 1, rs));
    }
    GH_CUDA_TRY(cudaEventRecord(ev_ready[b], rs));
    return GH_OK;
  };
  GH_TRY(recompute(nseg - 1));
  for (int64_t s = nseg - 1; s >= 0; s--) {
    const int b = (int)(s & 1);
    GH_CUDA_TRY(cudaStreamWaitEvent(st, ev_ready[b], 0));
    if (s >= 1) {
      // buffer (s-1)&1 was last read by the backward of segment s+1
      if (s + 1 < nseg) GH_CUDA_TRY(cudaStreamWaitEvent(rs, ev_free, 0));
      GH_TRY(recompute(s - 1));
    }
    GH_TRY(backward_steps(ws, (const double*)ws.chain_x[b].ptr, (const double*)ws.chain_v[b].ptr, mass, n, seg[s],
                          dt, eps, precision, xbar, vbar, mbar, st));
    GH_CUDA_TRY(cudaEventRecord(ev_free, st));
  }
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
