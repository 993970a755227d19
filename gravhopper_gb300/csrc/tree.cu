// Barnes-Hut octree on the GPU with the reference's exact cell geometry and
// opening decisions (gravhopper/_jbgrav.c:360-541, 737-806).
//
// Build (every force evaluation):
//   1. bounding box and root cell with the reference's boxsize rule (_jbgrav.c:747-775);
//   2. per-particle octant keys: at each level the octant is (x>cx, y>cy, z>cz) and the
//      child centre is c + (+-0.5*halfsize), the same FP64 recurrence as
//      gravoct_calc_subnode / gravoct_add_particle (_jbgrav.c:403-428, 453-462); read
//      off the bits of (p - c_0)/size wherever that provably gives the same decisions.
//      21 levels per 64-bit word, MSB first, digit = x | y<<1 | z<<2 (the reference's
//      branch number, _jbgrav.c:441-450), so key order is depth-first order with
//      children in branch order 0..7.  The number of words grows until no two
//      particles share a full key (coincident particles end with GH_ERR_DEPTH);
//   3. sort of the keys: a radix sort of the first word, then runs of equal first
//      words ordered by the other words (a full multi-word radix sort for long runs);
//   4. the node set of the reference's uncompressed octree (every cell that holds a
//      particle and whose parent holds at least two, single-child chains included)
//      laid out in depth-first preorder with skip ("next") indices, from the common
//      prefix lengths of neighbouring keys;
//   5. monopoles: leaves take the particle's position and mass exactly
//      (gravoct_finalize, _jbgrav.c:467-483); a cell holds a contiguous range of the
//      key-ordered particles, so its mass and first moment are differences of exact
//      192-bit fixed-point prefix sums, rounded to FP64 once (the reference rounds
//      after every particle it adds, in insertion order, so the last bits of an
//      internal COM can differ), and the centre of mass is first moment over mass.
// Walk: one warp per 32 consecutive targets in key order.  Each lane applies the
// reference's test "leaf or size/|center - x| < theta" (_jbgrav.c:496-502) to every
// cell its own traversal reaches; the warp visits the union of those cells in
// preorder, a lane skipping the subtrees it accepted.  The test is decided in FP32
// from hi/lo split coordinates with a 1e-4 relative margin; inside the margin it is
// recomputed with the reference's FP64 operations, so every lane takes exactly the
// reference's decisions.  Accepted cells contribute (COM - x) m / (r^2 + eps^2)^1.5 in
// FP64, with the reference's zero for r^2 + eps^2 == 0 (_jbgrav.c:514-520).
#include <cmath>
#include <mutex>

#include "direct.cuh"
#include "engine.h"
#include "fixed192.cuh"
#include "sort.cuh"

namespace gh {

constexpr int KEY_LEVELS = 21;
constexpr int KEY_BITS = 63;
constexpr int TREE_MIN_WORDS = 2;
constexpr int TREE_MAX_WORDS = 6;
constexpr double TREE_MARGIN = 1e-4;

struct TreeRoot {
  double c[3];
  double size;
  double inv;           // RN(1 / size)
  long long margin;     // 0: fast keys allowed; -1: the FP64 recurrence for every particle
  int bad;              // a particle position or mass is NaN or infinite
  int lsb_m, lsb_f;     // fixed-point units (2^lsb) of the mass and first-moment sums
};

// ---------------------------------------------------------------------------
// 1. Bounding box and root cell
// ---------------------------------------------------------------------------
constexpr int BB_THREADS = 256;
constexpr int BB_BLOCKS = 304;

// Per block: the box (min xyz, max xyz), whether any position or mass is not finite
// (the reference's insert never terminates on such particles) and the largest |mass|,
// 8 doubles.
constexpr int BB_PART = 8;

__global__ void __launch_bounds__(BB_THREADS)
    bbox_partial_kernel(const double* __restrict__ pos, const double* __restrict__ mass, int64_t n,
                        double* __restrict__ part) {
  __shared__ double s_mn[3][BB_THREADS], s_mx[3][BB_THREADS];
  __shared__ double s_m[BB_THREADS];
  double mn[3], mx[3], mmax = 0.0;
  bool have = false, bad = false;
  for (int64_t i = (int64_t)blockIdx.x * BB_THREADS + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * BB_THREADS) {
    const double mi = mass[i];
    bad = bad || !isfinite(mi);
    mmax = fmax(mmax, fabs(mi));
#pragma unroll
    for (int k = 0; k < 3; k++) {
      double q = pos[3 * i + k];
      bad = bad || !isfinite(q);
      if (!have) {
        mn[k] = mx[k] = q;
      } else {
        if (q < mn[k]) mn[k] = q;
        if (q > mx[k]) mx[k] = q;
      }
    }
    have = true;
  }
  if (!have) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      mn[k] = __longlong_as_double(0x7ff0000000000000ll);   // +inf
      mx[k] = __longlong_as_double(0xfff0000000000000ll);   // -inf
    }
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    s_mn[k][threadIdx.x] = mn[k];
    s_mx[k][threadIdx.x] = mx[k];
  }
  s_m[threadIdx.x] = mmax;
  bad = __syncthreads_or(bad);
  for (int s = BB_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        double a = s_mn[k][threadIdx.x + s], b = s_mx[k][threadIdx.x + s];
        if (a < s_mn[k][threadIdx.x]) s_mn[k][threadIdx.x] = a;
        if (b > s_mx[k][threadIdx.x]) s_mx[k][threadIdx.x] = b;
      }
      s_m[threadIdx.x] = fmax(s_m[threadIdx.x], s_m[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      part[BB_PART * blockIdx.x + k] = s_mn[k][0];
      part[BB_PART * blockIdx.x + 3 + k] = s_mx[k][0];
    }
    part[BB_PART * blockIdx.x + 6] = bad ? 1.0 : 0.0;
    part[BB_PART * blockIdx.x + 7] = s_m[0];
  }
}

// treeforce_workhorse, _jbgrav.c:764-772: boxsize = extent_x + eps, replaced by
// extent_i + eps when extent_i (without eps) exceeds it; centre = bbox midpoint.
// One warp folds the per-block partial boxes.
//
// Fast keys.  The reference's cell centres follow c_{l+1} = RN(c_l +- size 2^-(l+2)).
// Along a particle's own path the level-(l+1) centre lies within size 2^-(l+2) of p,
// so that rounding moves it by at most 2^-53 (|p| + size 2^-(l+2)), and after 42
// levels the centre is within E_c = 2^-53 (42 |p| + size/2) of the exact dyadic
// centre (per axis).  With t = (p - c_0) / size + 1/2 computed as
// fma(p - c_0, RN(1/size), 1/2) (error below 2^-52), each of the first 42 octant
// decisions "p > c_l" equals the bit of t at that level unless t lies within
// E_c / size + 2^-52 of a multiple of 2^-42.  keys_kernel keeps that window, doubled,
// in units of 2^-63; particles inside it take the reference's FP64 recurrence, as do
// all particles when the box size is outside [2^-900, 2^900] (margin -1).
__global__ void root_kernel(const double* __restrict__ part, int nb, double eps, TreeRoot* __restrict__ root) {
  if (blockIdx.x) return;
  const int lane = threadIdx.x;
  const double inf = __longlong_as_double(0x7ff0000000000000ll);
  double mn[3] = {inf, inf, inf}, mx[3] = {-inf, -inf, -inf}, mmax = 0.0;
  bool bad = false;
  for (int b = lane; b < nb; b += 32) {
    for (int k = 0; k < 3; k++) {
      const double a = part[BB_PART * b + k], c = part[BB_PART * b + 3 + k];
      if (a < mn[k]) mn[k] = a;
      if (c > mx[k]) mx[k] = c;
    }
    bad = bad || part[BB_PART * b + 6] != 0.0;
    mmax = fmax(mmax, part[BB_PART * b + 7]);
  }
  bad = __any_sync(0xffffffffu, bad);
  for (int o = 16; o > 0; o >>= 1) mmax = fmax(mmax, __shfl_xor_sync(0xffffffffu, mmax, o));
  for (int o = 16; o > 0; o >>= 1)
    for (int k = 0; k < 3; k++) {
      const double a = __shfl_xor_sync(0xffffffffu, mn[k], o), c = __shfl_xor_sync(0xffffffffu, mx[k], o);
      if (a < mn[k]) mn[k] = a;
      if (c > mx[k]) mx[k] = c;
    }
  if (lane) return;
  double bs = dadd(dsub(mx[0], mn[0]), eps);
  for (int k = 1; k < 3; k++)
    if (dsub(mx[k], mn[k]) > bs) bs = dadd(dsub(mx[k], mn[k]), eps);
  double amax = 0.0;
  for (int k = 0; k < 3; k++) {
    root->c[k] = dmul(0.5, dadd(mn[k], mx[k]));
    amax = fmax(amax, fabs(root->c[k]));
  }
  root->size = bs;
  root->bad = bad ? 1 : 0;
  // fixed-point units: |m| < 2^Bm and |m x| < 2^(Bm + Bx + 1) (the product's rounding
  // included), headroom for 2^24 particles (fixed192.cuh); floored so that sums of
  // exotic tiny inputs stay normal doubles
  if (!bad) {
    double xmax = 0.0;
    for (int k = 0; k < 3; k++) xmax = fmax(xmax, fmax(fabs(mn[k]), fabs(mx[k])));
    const int bm = fx::bound_exponent(mmax), bx = fx::bound_exponent(xmax);
    root->lsb_m = max(bm - fx::FX_HEADROOM, -1000);
    root->lsb_f = max(bm + bx + 1 - fx::FX_HEADROOM, -1000);
  } else {
    root->lsb_m = root->lsb_f = 0;
  }
  root->inv = ddiv(1.0, bs);
  root->margin = (bs > 0x1p-900 && bs < 0x1p+900 && amax < 0x1p+900) ? 0 : -1;
}

// ---------------------------------------------------------------------------
// 2. Octant keys
// ---------------------------------------------------------------------------
constexpr int TREE_MAX_LEVELS = KEY_LEVELS * TREE_MAX_WORDS;

// Spreads the low 21 bits of v to every third bit (bit b to bit 3b).
__device__ __forceinline__ uint64_t spread3(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x001f00000000ffffull;
  v = (v | (v << 16)) & 0x001f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

__device__ __forceinline__ unsigned lane_mask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Appends i to list (warp-aggregated) where `need`; every lane of the warp calls it.
__device__ __forceinline__ void warp_append(bool need, int64_t i, int* __restrict__ list, int* __restrict__ count) {
  const unsigned mask = __ballot_sync(0xffffffffu, need);
  if (!mask) return;
  int base = 0;
  if ((threadIdx.x & 31) == 0) base = atomicAdd(count, __popc(mask));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (need) list[base + __popc(mask & lane_mask_lt())] = (int)i;
}

// Fast keys where the decisions are provably the recurrence's (see root_kernel);
// the other particles are listed for keys_exact_kernel, so that the FP64 recurrence
// runs on full warps.
__global__ void keys_kernel(const double* __restrict__ pos, int64_t n, const TreeRoot* __restrict__ root,
                            int words, uint64_t* __restrict__ keys, uint32_t* __restrict__ idx,
                            int* __restrict__ list, int* __restrict__ count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool need = false;
  if (i < n) {
    idx[i] = (uint32_t)i;
    need = true;
    if (root->margin >= 0 && words == 2) {
      uint64_t T[3];
      bool ok = true;
      const double inv = root->inv;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const double p = pos[3 * i + k];
        const double t = fma(dsub(p, root->c[k]), inv, 0.5);
        T[k] = t >= 1.0 ? (1ull << 63) : (t > 0.0 ? (uint64_t)(t * 0x1p63) : 0ull);
        // 2 * 2^63 * (E_c / size + 2^-52) + slack, in FP32 (a bound, not a value)
        const float mf = fmaf(86016.f * 1.01f * fabsf((float)p), (float)inv, 5200.f);
        const uint64_t r = T[k] & ((1ull << 21) - 1);
        ok = ok && mf < 1048576.f && r > (uint64_t)mf && r < (1ull << 21) - (uint64_t)mf;
      }
      if (ok) {
        keys[i] = spread3(T[0] >> 42) | (spread3(T[1] >> 42) << 1) | (spread3(T[2] >> 42) << 2);
        keys[n + i] = spread3(T[0] >> 21) | (spread3(T[1] >> 21) << 1) | (spread3(T[2] >> 21) << 2);
        need = false;
      }
    }
  }
  warp_append(need, i, list, count);
}

// The reference's recurrence (gravoct_calc_subnode, _jbgrav.c:441-462) for the
// listed particles.
__global__ void keys_exact_kernel(const double* __restrict__ pos, int64_t n, const TreeRoot* __restrict__ root,
                                  int words, uint64_t* __restrict__ keys, const int* __restrict__ list,
                                  const int* __restrict__ count) {
  // child-centre offsets 0.5 * halfsize = size 2^-(l+2), exact scalings of the root size
  __shared__ double offs[TREE_MAX_LEVELS];
  const double S = root->size;
  for (int l = threadIdx.x; l < TREE_MAX_LEVELS; l += blockDim.x)
    offs[l] = dmul(S, __longlong_as_double((long long)(1023 - (l + 2)) << 52));
  __syncthreads();
  const int cnt = *count;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += gridDim.x * blockDim.x) {
    const int64_t i = list[q];
    const double p0 = pos[3 * i], p1 = pos[3 * i + 1], p2 = pos[3 * i + 2];
    double c0 = root->c[0], c1 = root->c[1], c2 = root->c[2];
    for (int w = 0; w < words; w++) {
      uint64_t k = 0;
#pragma unroll 3
      for (int l = 0; l < KEY_LEVELS; l++) {
        const double off = offs[w * KEY_LEVELS + l];
        const unsigned g0 = p0 > c0, g1 = p1 > c1, g2 = p2 > c2;
        c0 = g0 ? dadd(c0, off) : dsub(c0, off);
        c1 = g1 ? dadd(c1, off) : dsub(c1, off);
        c2 = g2 ? dadd(c2, off) : dsub(c2, off);
        k = (k << 3) | (uint64_t)(g0 | (g1 << 1) | (g2 << 2));
      }
      keys[(int64_t)w * n + i] = k;
    }
  }
}

// Keys of target points (two words, 42 levels of the sources' root cell; points
// outside it clamped to its faces) for the walk's order only: warps that hold
// neighbouring targets visit nearly the same cells.  Any order gives each target the
// same decisions and interactions, so these keys need not be the reference's.
__global__ void target_keys_kernel(const double* __restrict__ tpos, int64_t nt, const TreeRoot* __restrict__ root,
                                   uint64_t* __restrict__ keys, uint32_t* __restrict__ idx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  uint64_t T[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double t = fma(tpos[3 * i + k] - root->c[k], root->inv, 0.5);
    T[k] = t >= 1.0 ? ((1ull << 63) - 1) : (t > 0.0 ? (uint64_t)(t * 0x1p63) : 0ull);  // NaN: 0
  }
  keys[i] = spread3(T[0] >> 42) | (spread3(T[1] >> 42) << 1) | (spread3(T[2] >> 42) << 2);
  keys[nt + i] = spread3(T[0] >> 21) | (spread3(T[1] >> 21) << 1) | (spread3(T[2] >> 21) << 2);
  idx[i] = (uint32_t)i;
}

__device__ __forceinline__ int key_lcp(const uint64_t* __restrict__ keys, int words, int64_t n, int64_t a,
                                       int64_t b) {
  for (int w = 0; w < words; w++) {
    uint64_t x = keys[(int64_t)w * n + a] ^ keys[(int64_t)w * n + b];
    if (x) return w * KEY_LEVELS + (__clzll((long long)x) - 1) / 3;
  }
  return words * KEY_LEVELS;
}

__device__ __forceinline__ unsigned key_digit(const uint64_t* __restrict__ keys, int64_t n, int64_t i, int level) {
  const int w = level / KEY_LEVELS, l = level - w * KEY_LEVELS;
  return (unsigned)((keys[(int64_t)w * n + i] >> (3 * (KEY_LEVELS - 1 - l))) & 7u);
}

// ---------------------------------------------------------------------------
// 3. Sort: the first key word with a radix sort, then the rare runs of equal first
//    words ordered by the remaining words in place.  Equal full keys make the build
//    widen the keys and start again, so the final order is the full-key order.
// ---------------------------------------------------------------------------
constexpr int TIE_MAX_RUN = 256;  // longer runs of equal first words: full radix sort

// Brings key words 1.. into the order of the sorted first word: out[w][i] = in[w][idx[i]].
__global__ void gather_words_kernel(const uint64_t* __restrict__ kin, uint64_t* __restrict__ kout, int words,
                                    int64_t n, const uint32_t* __restrict__ idx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t src = idx[i];
  for (int w = 1; w < words; w++) kout[(int64_t)w * n + i] = kin[(int64_t)w * n + src];
}

__device__ __forceinline__ bool tied_first_word(const uint64_t* __restrict__ k0, int64_t n, int64_t i) {
  const uint64_t k = k0[i];
  return (i > 0 && k0[i - 1] == k) || (i + 1 < n && k0[i + 1] == k);
}

// Each particle in a run of equal first words takes its rank within the run by
// (words 1.., original index) and writes its key and index to that slot of the
// temporaries; flags[2] marks a run longer than TIE_MAX_RUN.
__global__ void tie_rank_kernel(const uint64_t* __restrict__ keys, int words, int64_t n,
                                const uint32_t* __restrict__ idx, uint64_t* __restrict__ kt,
                                uint32_t* __restrict__ it, int* __restrict__ flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !tied_first_word(keys, n, i)) return;
  const uint64_t k = keys[i];
  if ((i >= TIE_MAX_RUN && keys[i - TIE_MAX_RUN] == k) || (i + TIE_MAX_RUN < n && keys[i + TIE_MAX_RUN] == k)) {
    atomicOr(&flags[2], 1);  // sorted keys: the run is longer than TIE_MAX_RUN
    return;
  }
  int64_t s = i, e = i + 1;
  while (s > 0 && keys[s - 1] == k) {
    if (i - --s >= TIE_MAX_RUN) {
      atomicOr(&flags[2], 1);
      return;
    }
  }
  while (e < n && keys[e] == k) {
    if (++e - i > TIE_MAX_RUN) {
      atomicOr(&flags[2], 1);
      return;
    }
  }
  const uint32_t me = idx[i];
  int64_t r = 0;
  for (int64_t j = s; j < e; j++) {
    if (j == i) continue;
    int c = 0;  // -1: j before i, +1: j after i
    for (int w = 1; w < words && c == 0; w++) {
      const uint64_t a = keys[(int64_t)w * n + j], b = keys[(int64_t)w * n + i];
      c = a < b ? -1 : (a > b ? 1 : 0);
    }
    if (c < 0 || (c == 0 && idx[j] < me)) r++;
  }
  for (int w = 1; w < words; w++) kt[(int64_t)w * n + s + r] = keys[(int64_t)w * n + i];
  it[s + r] = me;
}

__global__ void tie_copy_kernel(uint64_t* __restrict__ keys, int words, int64_t n, uint32_t* __restrict__ idx,
                                const uint64_t* __restrict__ kt, const uint32_t* __restrict__ it) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !tied_first_word(keys, n, i)) return;
  for (int w = 1; w < words; w++) keys[(int64_t)w * n + i] = kt[(int64_t)w * n + i];
  idx[i] = it[i];
}

// flags[0]: two particles share a full key; flags[1]: deepest leaf level.
__global__ void lcp_kernel(const uint64_t* __restrict__ keys, int words, int64_t n, int* __restrict__ lp,
                           int* __restrict__ flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  if (i == 0 || i == n) {
    lp[i] = -1;
    return;
  }
  int l = key_lcp(keys, words, n, i - 1, i);
  lp[i] = l;
  if (l >= words * KEY_LEVELS) atomicOr(&flags[0], 1);
}

// Leaf level d_i = 1 + max(common prefix with either neighbour); particle i opens
// the cells at levels lp[i]+1 .. d_i (count d_i - lp[i]).
__global__ void count_kernel(const int* __restrict__ lp, int64_t n, int* __restrict__ cnt,
                             int* __restrict__ depth, int* __restrict__ flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int a = lp[i], b = lp[i + 1];
  const int d = 1 + (a > b ? a : b);
  depth[i] = d;
  cnt[i] = d - a;
  atomicMax(&flags[1], d);
}

// ---------------------------------------------------------------------------
// 4. Nodes in preorder
// ---------------------------------------------------------------------------
// The walk's per-node record, 48 bytes (two 32-byte sectors) per visited cell.  A
// leaf's "centre" is its particle's position and its offset is zero, so the offset
// from the target computed for the opening test is, plus O, the offset of the centre
// of mass: accepted cells are at least size/theta away, so O's FP32 rounding is below
// 2^-24 theta of the distance.
struct __align__(16) WalkRec {
  float4 A;   // (cx_hi, cy_hi, cz_hi, size^2)        FP32 opening prefilter
  float4 L;   // (cx_lo, cy_lo, cz_lo, next as bits)   FP32 residuals + skip index
  float4 O;   // (com - c as FP32, mass)              mixed-precision interaction
};

struct NodeArrays {
  WalkRec* R;    // walk records (A, L, O)
  dvec4* C;      // (cx, cy, cz, size)                    exact opening test (internal cells)
  dvec4* M;      // (comx, comy, comz, mass)              interaction
};

// Exact prefix sums over the key-ordered particles: mass and first moment x, y, z.
struct FxMoments {
  fx::I192 c[4];
};
constexpr int MS_THREADS = 256, MS_ITEMS = 8, MS_TILE = MS_THREADS * MS_ITEMS;

__device__ __forceinline__ void fxm_add(FxMoments& a, const FxMoments& b) {
#pragma unroll
  for (int k = 0; k < 4; k++) a.c[k] = fx::add(a.c[k], b.c[k]);
}

__device__ __forceinline__ FxMoments fxm_zero() {
  FxMoments r;
#pragma unroll
  for (int k = 0; k < 4; k++) r.c[k] = fx::zero();
  return r;
}

// Prefix over the first j key-ordered particles (j <= n): the tile's prefix plus the
// prefix within the tile.
__device__ __forceinline__ FxMoments fxm_prefix(const FxMoments* __restrict__ local,
                                                const FxMoments* __restrict__ tiles, int64_t j, int64_t n) {
  if (j >= n) return tiles[(n + MS_TILE - 1) / MS_TILE];
  FxMoments r = tiles[j / MS_TILE];
  fxm_add(r, local[j]);
  return r;
}

__device__ __forceinline__ float f32_hi(double v) { return (float)v; }
__device__ __forceinline__ float f32_lo(double v, float hi) { return (float)(v - (double)hi); }

// First particle after i that shares fewer than L leading digits with it: a short
// scan of the neighbour prefixes, then a binary search on the keys.
__device__ __forceinline__ int64_t cell_end(const uint64_t* __restrict__ keys, int words, int64_t n,
                                            const int* __restrict__ lp, int64_t i, int L) {
  int64_t j = i + 1;
  for (int s = 0; s < 16; s++, j++)
    if (lp[j] < L) return j;  // lp[n] = -1 ends the scan
  int64_t a = j - 1, b = n - 1;  // a shares >= L digits with i
  // gallop: most cells are small, so bracket the end before bisecting
  for (int64_t step = 32; a + step < b; step *= 2) {
    if (key_lcp(keys, words, n, i, a + step) < L) {
      b = a + step - 1;
      break;
    }
    a += step;
  }
  while (a < b) {
    const int64_t mid = (a + b + 1) >> 1;
    if (key_lcp(keys, words, n, i, mid) >= L)
      a = mid;
    else
      b = mid - 1;
  }
  return a + 1;
}

// Particle i opens the cells at levels lo = lp[i]+1 .. d (its leaf), nodes
// base[i] .. base[i] + d - lo in preorder.  nodes_kernel writes the leaf: the
// particle's position as its centre, its mass, its skip index (gravoct_finalize,
// _jbgrav.c:467-483: a leaf's centre of mass is its particle), and lists the
// particles that open internal cells and the internal cells themselves;
// cell_centres_kernel gives those cells their centre from the reference's FP64
// recurrence along the particle's digits (gravoct_add_particle, _jbgrav.c:403-428),
// cells_kernel their skip index and their monopole.  A leaf is always accepted by the
// walk, so it needs no geometric centre.
__global__ void nodes_kernel(int64_t n, const int* __restrict__ lp, const int* __restrict__ depth,
                             const int* __restrict__ base, const uint32_t* __restrict__ perm,
                             const double* __restrict__ pos, const double* __restrict__ mass, NodeArrays na,
                             int nnodes, int* __restrict__ list, int* __restrict__ count,
                             int2* __restrict__ cells, int* __restrict__ ncells) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool need = false;
  int ncell = 0, k0 = 0;  // this particle's internal cells: nodes k0 .. k0 + ncell - 1
  if (i < n) {
    const int lo = lp[i] + 1, d = depth[i];
    const int k = base[i] + (d - lo);
    const int next = i + 1 < n ? base[i + 1] : nnodes;
    const int64_t p = perm[i];
    const double m = mass[p];
    const double x = pos[3 * p], y = pos[3 * p + 1], z = pos[3 * p + 2];
    na.M[k] = make_dvec4(x, y, z, m);
    const float hx = (float)x, hy = (float)y, hz = (float)z;
    na.R[k].A = make_float4(hx, hy, hz, 0.f);
    na.R[k].L = make_float4(f32_lo(x, hx), f32_lo(y, hy), f32_lo(z, hz), __int_as_float(next));
    na.R[k].O = make_float4(0.f, 0.f, 0.f, (float)m);
    need = d > lo;
    ncell = d - lo;
    k0 = base[i];
  }
  warp_append(need, i, list, count);
  // the internal cells, one (cell, opener) entry each, for cells_kernel
  const int lane = threadIdx.x & 31;
  int incl = ncell;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  int first = 0;
  if (lane == 31 && incl > 0) first = atomicAdd(ncells, incl);
  first = __shfl_sync(0xffffffffu, first, 31) + incl - ncell;
  for (int j = 0; j < ncell; j++) cells[first + j] = make_int2(k0 + j, (int)i);
}

__device__ __forceinline__ double rcp_f64(double m);

// Centres of the internal cells from the reference's FP64 recurrence along each
// opener's digits (gravoct_add_particle, _jbgrav.c:403-428): C[k] = (centre, size).
// Only the recurrence runs here, so its FP64 adds keep most lanes of a warp busy; the
// rest of each cell is cells_kernel's, one thread per cell.
__global__ void cell_centres_kernel(const uint64_t* __restrict__ keys, int words, int64_t n,
                                    const int* __restrict__ lp, const int* __restrict__ depth,
                                    const int* __restrict__ base, const TreeRoot* __restrict__ root, NodeArrays na,
                                    const int* __restrict__ list, const int* __restrict__ count) {
  __shared__ double offs[TREE_MAX_LEVELS];  // size 2^-(L+2), exact
  const double S = root->size;
  for (int l = threadIdx.x; l < TREE_MAX_LEVELS; l += blockDim.x)
    offs[l] = dmul(S, __longlong_as_double((long long)(1023 - (l + 2)) << 52));
  __syncthreads();
  const int cnt = *count;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += gridDim.x * blockDim.x) {
    const int64_t i = list[q];
    const int lo = lp[i] + 1, d = depth[i];
    const int k0 = base[i];
    const uint64_t kw0 = keys[i], kw1 = words > 1 ? keys[n + i] : 0ull;  // digits of the first 42 levels
    double c[3] = {root->c[0], root->c[1], root->c[2]};
    for (int L = 0; L < d; L++) {
      if (L >= lo)
        na.C[k0 + (L - lo)] = make_dvec4(c[0], c[1], c[2], dmul(S, __longlong_as_double((long long)(1023 - L) << 52)));
      if (L + 1 < d) {
        const unsigned g = L < KEY_LEVELS       ? (unsigned)(kw0 >> (3 * (KEY_LEVELS - 1 - L))) & 7u
                           : L < 2 * KEY_LEVELS ? (unsigned)(kw1 >> (3 * (2 * KEY_LEVELS - 1 - L))) & 7u
                                                : key_digit(keys, n, i, L);
        const double off = offs[L];
#pragma unroll
        for (int r = 0; r < 3; r++) c[r] = ((g >> r) & 1u) ? dadd(c[r], off) : dsub(c[r], off);
      }
    }
  }
}

// One internal cell per thread (the (cell, opener) list of nodes_kernel): its skip
// index, its walk record from the centre, and its monopole.  Cell k of opener i is at
// level L = lp[i] + 1 + (k - base[i]) and holds the key-ordered particles [i, end).
__global__ void cells_kernel(const uint64_t* __restrict__ keys, int words, int64_t n, const int* __restrict__ lp,
                             const int* __restrict__ base, const TreeRoot* __restrict__ root, NodeArrays na,
                             int nnodes, const int2* __restrict__ cells, int ncells,
                             const FxMoments* __restrict__ fx_local, const FxMoments* __restrict__ fx_tiles) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ncells) return;
  const int2 e = cells[q];
  const int k = e.x;
  const int64_t i = e.y;
  const int L = lp[i] + 1 + (k - base[i]);
  const int lsb_m = root->lsb_m, lsb_f = root->lsb_f;
  const dvec4 C = na.C[k];
  const int64_t end = cell_end(keys, words, n, lp, i, L);
  const int next = end < n ? base[end] : nnodes;
  const double c[3] = {C.x, C.y, C.z};
  float4 A, Lo;
  A.x = f32_hi(c[0]);
  A.y = f32_hi(c[1]);
  A.z = f32_hi(c[2]);
  A.w = (float)dmul(C.w, C.w);
  Lo.x = f32_lo(c[0], A.x);
  Lo.y = f32_lo(c[1], A.y);
  Lo.z = f32_lo(c[2], A.z);
  Lo.w = __int_as_float(next);
  na.R[k].A = A;
  na.R[k].L = Lo;
  // monopole of particles [i, end): exact sums, one rounding each, then
  // firstmoment / mass (_jbgrav.c:478) with a Newton-refined reciprocal
  const FxMoments Pi = fxm_prefix(fx_local, fx_tiles, i, n);
  const FxMoments Pe = fxm_prefix(fx_local, fx_tiles, end, n);
  const double cm = fx::to_double(fx::sub(Pe.c[0], Pi.c[0]), lsb_m);
  const double r = rcp_f64(cm);
  double com[3];
#pragma unroll
  for (int a2 = 0; a2 < 3; a2++) com[a2] = dmul(fx::to_double(fx::sub(Pe.c[a2 + 1], Pi.c[a2 + 1]), lsb_f), r);
  na.M[k] = make_dvec4(com[0], com[1], com[2], cm);
  na.R[k].O = make_float4((float)dsub(com[0], c[0]), (float)dsub(com[1], c[1]), (float)dsub(com[2], c[2]),
                          (float)cm);
}

// ---------------------------------------------------------------------------
// 5. Exact prefix sums of the monopole moments over the key-ordered particles
// ---------------------------------------------------------------------------
// The particles of a cell are a contiguous range [first, end) of the key order, so
// its mass and first moment (m_j x_j, the reference's FP64 products,
// gravoct_add_particle, _jbgrav.c:396-398) are differences of prefix sums.  The sums
// are exact 192-bit fixed-point integers (fixed192.cuh): their values do not depend on
// the order of addition, and each cell's is rounded to FP64 once.

// 1/m from the hardware approximation and two Newton steps y <- y + y (1 - m y).
__device__ __forceinline__ double rcp_f64(double m) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(m));
#pragma unroll
  for (int it = 0; it < 2; it++) y = fma(y, fma(-m, y, 1.0), y);
  return y;
}

__device__ __forceinline__ FxMoments particle_moments(const double* __restrict__ pos,
                                                      const double* __restrict__ mass, int64_t p, int lsb_m,
                                                      int lsb_f) {
  const double m = mass[p];
  FxMoments r;
  r.c[0] = fx::from_double(m, lsb_m);
#pragma unroll
  for (int a = 0; a < 3; a++) r.c[a + 1] = fx::from_double(dmul(m, pos[3 * p + a]), lsb_f);
  return r;
}

// Exclusive scan of the threads' totals within a block of MS_THREADS; returns the
// thread's exclusive prefix.
__device__ __forceinline__ FxMoments fxm_block_exclusive(const FxMoments& tot) {
  __shared__ FxMoments warp_tot[MS_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  FxMoments inc = tot;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    FxMoments y;
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
      for (int w = 0; w < 3; w++) y.c[k].w[w] = __shfl_up_sync(0xffffffffu, inc.c[k].w[w], d);
    if (lane >= d) fxm_add(inc, y);
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  FxMoments before = fxm_zero();
  for (int w = 0; w < warp; w++) fxm_add(before, warp_tot[w]);
#pragma unroll
  for (int k = 0; k < 4; k++) before.c[k] = fx::add(before.c[k], fx::sub(inc.c[k], tot.c[k]));
  __syncthreads();  // warp_tot may be reused by the caller's next scan
  return before;
}

// Per tile of MS_TILE key-ordered particles: the prefix of every particle within its
// tile (fx_local) and the tile's total (fx_tiles[tile]).
__global__ void __launch_bounds__(MS_THREADS)
    moments_scan_kernel(const double* __restrict__ pos, const double* __restrict__ mass,
                        const uint32_t* __restrict__ perm, int64_t n, const TreeRoot* __restrict__ root,
                        FxMoments* __restrict__ fx_local, FxMoments* __restrict__ fx_tiles) {
  const int lsb_m = root->lsb_m, lsb_f = root->lsb_f;
  const int64_t j0 = (int64_t)blockIdx.x * MS_TILE + (int64_t)threadIdx.x * MS_ITEMS;
  // each item's moments are formed twice (for the thread's total, then for the running
  // prefix): measured cheaper than storing them and reading them back (1.22 against
  // 1.33 ms per build at N = 1M)
  FxMoments tot = fxm_zero();
  for (int r = 0; r < MS_ITEMS; r++)
    if (j0 + r < n) fxm_add(tot, particle_moments(pos, mass, perm[j0 + r], lsb_m, lsb_f));
  FxMoments run = fxm_block_exclusive(tot);
  for (int r = 0; r < MS_ITEMS; r++)
    if (j0 + r < n) {
      fx_local[j0 + r] = run;
      fxm_add(run, particle_moments(pos, mass, perm[j0 + r], lsb_m, lsb_f));
    }
  if (threadIdx.x == MS_THREADS - 1) fx_tiles[blockIdx.x] = run;
}

// Exclusive scan of the tile totals in place; fx_tiles[ntiles] receives the total.
__global__ void __launch_bounds__(MS_THREADS) moments_tiles_kernel(FxMoments* __restrict__ fx_tiles, int64_t ntiles) {
  const int64_t per = (ntiles + MS_THREADS - 1) / MS_THREADS;
  const int64_t a = (int64_t)threadIdx.x * per;
  const int64_t b = a + per < ntiles ? a + per : ntiles;
  FxMoments tot = fxm_zero();
  for (int64_t t = a; t < b; t++) fxm_add(tot, fx_tiles[t]);
  FxMoments run = fxm_block_exclusive(tot);
  for (int64_t t = a; t < b; t++) {
    const FxMoments v = fx_tiles[t];
    fx_tiles[t] = run;
    fxm_add(run, v);
  }
  if (threadIdx.x == MS_THREADS - 1) fx_tiles[ntiles] = run;
}

// ---------------------------------------------------------------------------
// Walk
// ---------------------------------------------------------------------------
constexpr int TW_THREADS = 128;
constexpr int TW_MINB = 9;  // 56 registers, no spills: 36 warps per SM (measured fastest)

__device__ __forceinline__ double rsqrt_f64(double s) {
  double y;
  asm("rsqrt.approx.f64 %0, %1;" : "=d"(y) : "d"(s));
  // two Newton steps: y <- y + 0.5 y (1 - s y^2)
#pragma unroll
  for (int it = 0; it < 2; it++) {
    double e = fma(-s * y, y, 1.0);
    y = fma(0.5 * y, e, y);
  }
  return y;
}

// MIXED: accepted cells interact in FP32: the hi/lo split offset of the cell's
// centre (keeps ~2^-48 of |x|) plus the FP32 offset of its centre of mass; partial
// sums folded into a two-sum (hi, lo) accumulator every 32 interactions.  Otherwise
// FP64 with s^(-3/2) from the integer-pipe reciprocal square root (f64emu.cuh).
// The opening decisions are the same exact ones in both forms.
constexpr int TW_FOLD = 32;
// FP64: a lane's accepted cells wait in a FIFO of TW_FQ entries and are evaluated in
// rounds that run when at least TW_FQ_ROUND lanes have one waiting (or a FIFO is
// full), so the FP64 pipe (1/74 of the FP32 rate on GB300) issues fewer partly empty
// instructions; each lane still adds its interactions in visiting order.
constexpr int TW_FQ = 32;
constexpr int TW_FQ_ROUND = 28;
static_assert((TW_FQ & (TW_FQ - 1)) == 0, "the FIFO index wraps with a mask");

// One FP64 interaction: the cell's monopole (nM) with s^(-3/2) on the integer pipes,
// FP64 Newton steps outside the emulation's range.
template <bool GUARD>
__device__ __forceinline__ void walk_interact_f64(const dvec4* __restrict__ nM, int node, double p0, double p1,
                                                  double p2, double eps2, double& ax, double& ay, double& az) {
  const dvec4 M = nM[node];
  const double dx = M.x - p0, dy = M.y - p1, dz = M.z - p2;
  const double s = fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2)));
  if (!GUARD || s != 0.0) {
    double y3;
    if (!emu::rsqrt_cube(s, y3)) {
      const double y = rsqrt_f64(s);
      y3 = y * (y * y);
    }
    const double f = M.w * y3;
    ax = fma(f, dx, ax);
    ay = fma(f, dy, ay);
    az = fma(f, dz, az);
  }
}

template <bool GUARD, bool MIXED, bool STATS, class Epi>
__global__ void __launch_bounds__(TW_THREADS, TW_MINB)
    tree_walk_kernel(const WalkRec* __restrict__ nR, const dvec4* __restrict__ nC, const dvec4* __restrict__ nM,
                     int nnodes, const double* __restrict__ tpos, const uint32_t* __restrict__ order, int64_t nt,
                     double eps2, double theta, float th2_lo, float th2_hi, Epi epi,
                     unsigned long long* __restrict__ stats) {
  const int64_t slot = (int64_t)blockIdx.x * TW_THREADS + threadIdx.x;
  const bool valid = slot < nt;
  const int64_t t = valid ? (order ? (int64_t)order[slot] : slot) : 0;
  double p0 = 0.0, p1 = 0.0, p2 = 0.0;
  if (valid) {
    p0 = tpos[3 * t];
    p1 = tpos[3 * t + 1];
    p2 = tpos[3 * t + 2];
  }
  const float h0 = (float)p0, h1 = (float)p1, h2 = (float)p2;
  const float l0 = f32_lo(p0, h0), l1 = f32_lo(p1, h1), l2 = f32_lo(p2, h2);
  const f2 h01 = f2make(h0, h1), l01 = f2make(l0, l1);
  // d^2 below this needs the exact test: FP32 differences lose too much relative to
  // |x|, and FP32 stays in its normal range (with theta >= 1e-3 a cell whose size^2
  // is below that range is then accepted, as the exact test would)
  const float near2 = fmaxf(1e-18f * (h0 * h0 + h1 * h1 + h2 * h2), 1e-30f);
  const float eps2f = (float)eps2;
  double ax = 0.0, ay = 0.0, az = 0.0;
  float px = 0.f, py = 0.f, pz = 0.f;            // FP32 partial (MIXED)
  float hx = 0.f, hy = 0.f, hz = 0.f, qx = 0.f, qy = 0.f, qz = 0.f;  // two-sum hi, lo
  int pending = 0;
  __shared__ int fq[MIXED ? 1 : TW_FQ][TW_THREADS];  // FP64: this lane's accepted cells, FIFO
  int fq_head = 0, fq_n = 0;
  unsigned n_step = 0, n_visit = 0, n_inter = 0, n_exact = 0, n_leaf = 0, n_chain = 0;  // walk counters (STATS)
  int skip = valid ? 0 : 0x7fffffff;
  int node = __reduce_min_sync(0xffffffffu, skip);
  while (node < nnodes) {
    if (STATS) {
      n_step++;
      // a cell with one child cell: the child's subtree ends where the cell's does
      const int nxt = __float_as_int(nR[node].L.w);
      if (nxt != node + 1 && node + 1 < nnodes && __float_as_int(nR[node + 1].L.w) == nxt) n_chain++;
    }
    int lane_next = skip;
    if (node >= skip) {
      if (STATS) n_visit++;
      const float4 A = nR[node].A;
      const float4 Lo = nR[node].L;
      float4 O;  // loaded with the rest of the record: most visits are accepted
      if (MIXED) O = nR[node].O;
      const int nx = __float_as_int(Lo.w);
      bool accept = (nx == node + 1);  // leaf
      // (x, y) offsets as one f32x2 pair, z alone
      const f2 dxy = f2add(f2sub(f2make(A.x, A.y), h01), f2sub(f2make(Lo.x, Lo.y), l01));
      const float dz = (A.z - h2) + (Lo.z - l2);
      float dx, dy;
      f2split(dxy, dx, dy);
      if (!accept) {
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const float s2 = A.w;
        // d2 = inf (overflow) accepts, as the exact test does for so distant a cell
        const bool usable = d2 > near2;
        if (usable && s2 < th2_lo * d2) {
          accept = true;
        } else if (usable && s2 > th2_hi * d2) {
          accept = false;
        } else {
          // gravoct_calc_accel opening test with the reference's FP64 operations
          if (STATS) n_exact++;
          const dvec4 C = nC[node];
          const double e0 = dsub(C.x, p0), e1 = dsub(C.y, p1), e2 = dsub(C.z, p2);
          double nd = dmul(e0, e0);
          nd = dadd(nd, dmul(e1, e1));
          nd = dadd(nd, dmul(e2, e2));
          accept = ddiv(C.w, dsqrt(nd)) < theta;
        }
      }
      if (accept) {
        if (STATS) {
          n_inter++;
          if (nx == node + 1) n_leaf++;
        }
        if (MIXED) {
          float ex, ey;
          f2split(f2add(dxy, f2make(O.x, O.y)), ex, ey);
          const float ez = dz + O.z;
          const float s = fmaf(ex, ex, fmaf(ey, ey, fmaf(ez, ez, eps2f)));
          float r = rsqrt_approx(s);
          if (GUARD) r = s > 0.f ? r : 0.f;
          const float f = O.w * (r * (r * r));
          px = fmaf(f, ex, px);
          py = fmaf(f, ey, py);
          pz = fmaf(f, ez, pz);
        } else {
          fq[(fq_head + fq_n) & (TW_FQ - 1)][threadIdx.x] = node;  // evaluated in a later round
          fq_n++;
        }
        skip = nx;
        lane_next = nx;
      } else {
        lane_next = node + 1;
      }
    }
    if (!MIXED) {
      // a round of FP64 interactions when enough lanes have one waiting; a FIFO that
      // just became full forces one, so a FIFO never holds more than TW_FQ
      const unsigned waiting = __ballot_sync(0xffffffffu, fq_n > 0);
      if (__popc(waiting) >= TW_FQ_ROUND || __any_sync(0xffffffffu, fq_n == TW_FQ)) {
        if (fq_n > 0) {
          const int c = fq[fq_head][threadIdx.x];
          fq_head = (fq_head + 1) & (TW_FQ - 1);
          fq_n--;
          walk_interact_f64<GUARD>(nM, c, p0, p1, p2, eps2, ax, ay, az);
        }
      }
    }
    // fold the FP32 partials every TW_FOLD warp steps (at most one interaction per
    // target per step): a warp-uniform branch
    if (MIXED && ++pending == TW_FOLD) {
      float sx, ex;
      two_sum(hx, px, sx, ex);
      hx = sx;
      qx += ex;
      two_sum(hy, py, sx, ex);
      hy = sx;
      qy += ex;
      two_sum(hz, pz, sx, ex);
      hz = sx;
      qz += ex;
      px = py = pz = 0.f;
      pending = 0;
    }
    node = __reduce_min_sync(0xffffffffu, lane_next);
  }
  if (!MIXED) {
    while (fq_n > 0) {  // the cells still waiting, in order
      const int c = fq[fq_head][threadIdx.x];
      fq_head = (fq_head + 1) & (TW_FQ - 1);
      fq_n--;
      walk_interact_f64<GUARD>(nM, c, p0, p1, p2, eps2, ax, ay, az);
    }
  }
  if (STATS) {
    // one cell record read per warp step; the other counts summed over lanes
    n_visit = __reduce_add_sync(0xffffffffu, n_visit);
    n_inter = __reduce_add_sync(0xffffffffu, n_inter);
    n_exact = __reduce_add_sync(0xffffffffu, n_exact);
    n_leaf = __reduce_add_sync(0xffffffffu, n_leaf);
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(&stats[0], (unsigned long long)n_step);
      atomicAdd(&stats[1], (unsigned long long)n_visit);
      atomicAdd(&stats[2], (unsigned long long)n_inter);
      atomicAdd(&stats[3], (unsigned long long)n_exact);
      atomicAdd(&stats[4], (unsigned long long)n_leaf);
      atomicAdd(&stats[5], (unsigned long long)n_chain);
    }
  }
  if (MIXED) {
    ax = (double)hx + (double)qx + (double)px;
    ay = (double)hy + (double)qy + (double)py;
    az = (double)hz + (double)qz + (double)pz;
  }
  if (valid) epi(t, ax, ay, az);
}

// ---------------------------------------------------------------------------
// Workspace and host driver
// ---------------------------------------------------------------------------
struct TreeWS {
  Buffer part, root, keys, keys_tmp, idx, idx_tmp, rs, lp, cnt, depth, base, scan, flags;
  Buffer nA, nC, nM, fxl, fxt, xh[2];
  Buffer tkeys, tkeys_tmp, tidx, tidx_tmp, trs;  // target points' walk order
  Buffer list;                // particle lists: key fallbacks, then cell openers
  Buffer cells;               // (internal cell, opener) pairs
  int* host_flags = nullptr;  // pinned: the 8 device flags, nnodes, the root's non-finite flag
  int words = TREE_MIN_WORDS;
  int64_t full_sort_n = -1;  // particle count whose last build needed the full multi-word sort
};
static TreeWS g_tree[64];
static std::recursive_mutex g_tree_mu;

static NodeArrays node_arrays(TreeWS& ws) {
  NodeArrays na;
  na.R = (WalkRec*)ws.nA.ptr;
  na.C = (dvec4*)ws.nC.ptr;
  na.M = (dvec4*)ws.nM.ptr;
  return na;
}

struct BuiltTree {
  int nnodes = 0;
  int maxdepth = 0;
  const uint32_t* torder = nullptr;  // target points in key order (when sorted)
};

// Target points are walked in key order from this many on (below, the sort's fixed
// cost exceeds what the coherent warps save).
constexpr int64_t TGT_SORT_MIN = 8192;

static int tree_build(TreeWS& ws, const double* pos, const double* mass, int64_t n, double eps,
                      cudaStream_t st, BuiltTree* out, const double* tpos = nullptr, int64_t nt = 0) {
  Trace tr("tree build");
  const bool sort_targets = tpos != nullptr && nt >= TGT_SORT_MIN;
  if (sort_targets && nt > (1LL << 31))
    return set_error(GH_ERR_ARG, "tree: at most 2^31 target points (got %lld)", (long long)nt);
  // int32 node indices: at most 127 cells per particle
  if (n > (1LL << 24)) return set_error(GH_ERR_ARG, "tree: at most 16777216 particles (got %lld)", (long long)n);
  if (!ws.host_flags) GH_CUDA_TRY(cudaMallocHost((void**)&ws.host_flags, 16 * sizeof(int)));
  const int T = 256;
  // 1. root cell
  GH_TRY(ensure(ws.part, BB_BLOCKS * BB_PART * sizeof(double)));
  GH_TRY(ensure(ws.root, sizeof(TreeRoot)));
  int nb = (int)((n + BB_THREADS - 1) / BB_THREADS);
  if (nb > BB_BLOCKS) nb = BB_BLOCKS;
  bbox_partial_kernel<<<nb, BB_THREADS, 0, st>>>(pos, mass, n, (double*)ws.part.ptr);
  GH_LAUNCH_CHECK();
  root_kernel<<<1, 32, 0, st>>>((const double*)ws.part.ptr, nb, eps, (TreeRoot*)ws.root.ptr);
  GH_LAUNCH_CHECK();
  const TreeRoot* root = (const TreeRoot*)ws.root.ptr;
  const unsigned gn = (unsigned)((n + T - 1) / T), gn1 = (unsigned)((n + 1 + T - 1) / T);
  GH_TRY(ensure(ws.lp, (n + 1) * sizeof(int)));
  GH_TRY(ensure(ws.cnt, n * sizeof(int)));
  GH_TRY(ensure(ws.depth, n * sizeof(int)));
  GH_TRY(ensure(ws.base, (n + 1) * sizeof(int)));
  GH_TRY(ensure(ws.scan, scan_scratch_ints(n) * sizeof(int)));
  // flags: [0] full-key tie, [1] deepest level, [2] long run, [3] key fallbacks, [4] cell openers,
  // [5] a bounded wait in the sort gave up, [6] internal cells listed
  GH_TRY(ensure(ws.flags, 8 * sizeof(int)));
  GH_TRY(ensure(ws.list, n * sizeof(int)));
  GH_TRY(ensure(ws.idx, n * sizeof(uint32_t)));
  GH_TRY(ensure(ws.idx_tmp, n * sizeof(uint32_t)));
  GH_TRY(ensure(ws.rs, radix_scratch_words(n) * sizeof(uint32_t)));
  // 2-3. keys, sort, prefix structure; widen the keys while particles tie
  // A long run of equal first words usually recurs in the next build of the same
  // system (a stepping loop), so the full sort is kept for that particle count.
  bool full_sort = ws.full_sort_n == n;
  for (;;) {
    const int words = ws.words;
    GH_TRY(ensure(ws.keys, (size_t)words * n * sizeof(uint64_t)));
    GH_TRY(ensure(ws.keys_tmp, (size_t)words * n * sizeof(uint64_t)));
    uint64_t* keys = (uint64_t*)ws.keys.ptr;
    uint64_t* ktmp = (uint64_t*)ws.keys_tmp.ptr;
    uint32_t* idx = (uint32_t*)ws.idx.ptr;
    uint32_t* itmp = (uint32_t*)ws.idx_tmp.ptr;
    int* flags = (int*)ws.flags.ptr;
    GH_CUDA_TRY(cudaMemsetAsync(flags, 0, 8 * sizeof(int), st));
    keys_kernel<<<gn, T, 0, st>>>(pos, n, root, words, keys, idx, (int*)ws.list.ptr, flags + 3);
    GH_LAUNCH_CHECK();
    keys_exact_kernel<<<gn < 4 * 152 ? gn : 4 * 152, T, 0, st>>>(pos, n, root, words, keys, (const int*)ws.list.ptr,
                                                                flags + 3);
    GH_LAUNCH_CHECK();
    if (full_sort) {
      GH_TRY(radix_sort_keys(keys, idx, ktmp, itmp, words, KEY_BITS, n, (uint32_t*)ws.rs.ptr, st, flags + 5));
    } else {
      GH_TRY(radix_sort_keys(keys, idx, ktmp, itmp, 1, KEY_BITS, n, (uint32_t*)ws.rs.ptr, st, flags + 5));
      gather_words_kernel<<<gn, T, 0, st>>>(keys, ktmp, words, n, idx);
      GH_LAUNCH_CHECK();
      GH_CUDA_TRY(cudaMemcpyAsync(keys + n, ktmp + n, (size_t)(words - 1) * n * sizeof(uint64_t),
                                  cudaMemcpyDeviceToDevice, st));
      tie_rank_kernel<<<gn, T, 0, st>>>(keys, words, n, idx, ktmp, itmp, (int*)ws.flags.ptr);
      GH_LAUNCH_CHECK();
      tie_copy_kernel<<<gn, T, 0, st>>>(keys, words, n, idx, ktmp, itmp);
      GH_LAUNCH_CHECK();
    }
    if (inject_take(GH_INJECT_TREE_WAIT))  // test hook: as if a look-back wait had run out
      GH_CUDA_TRY(cudaMemsetAsync(flags + 5, 1, 1, st));
    lcp_kernel<<<gn1, T, 0, st>>>(keys, words, n, (int*)ws.lp.ptr, (int*)ws.flags.ptr);
    GH_LAUNCH_CHECK();
    count_kernel<<<gn, T, 0, st>>>((const int*)ws.lp.ptr, n, (int*)ws.cnt.ptr, (int*)ws.depth.ptr,
                                   (int*)ws.flags.ptr);
    GH_LAUNCH_CHECK();
    GH_TRY(exclusive_scan_i32((const int*)ws.cnt.ptr, (int*)ws.base.ptr, n, (int*)ws.scan.ptr, st));
    if (sort_targets) {  // the targets' walk order; its sort reports a given-up wait in flags[5] too
      GH_TRY(ensure(ws.tkeys, (size_t)2 * nt * sizeof(uint64_t)));
      GH_TRY(ensure(ws.tkeys_tmp, (size_t)2 * nt * sizeof(uint64_t)));
      GH_TRY(ensure(ws.tidx, (size_t)nt * sizeof(uint32_t)));
      GH_TRY(ensure(ws.tidx_tmp, (size_t)nt * sizeof(uint32_t)));
      GH_TRY(ensure(ws.trs, radix_scratch_words(nt) * sizeof(uint32_t)));
      target_keys_kernel<<<(unsigned)((nt + T - 1) / T), T, 0, st>>>(tpos, nt, root, (uint64_t*)ws.tkeys.ptr,
                                                                     (uint32_t*)ws.tidx.ptr);
      GH_LAUNCH_CHECK();
      GH_TRY(radix_sort_keys((uint64_t*)ws.tkeys.ptr, (uint32_t*)ws.tidx.ptr, (uint64_t*)ws.tkeys_tmp.ptr,
                             (uint32_t*)ws.tidx_tmp.ptr, 2, KEY_BITS, nt, (uint32_t*)ws.trs.ptr, st, flags + 5));
      out->torder = (const uint32_t*)ws.tidx.ptr;
    }
    GH_CUDA_TRY(cudaMemcpyAsync(ws.host_flags, ws.flags.ptr, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
    GH_CUDA_TRY(cudaMemcpyAsync(ws.host_flags + 8, (int*)ws.base.ptr + n, sizeof(int), cudaMemcpyDeviceToHost,
                                st));
    GH_CUDA_TRY(cudaMemcpyAsync(ws.host_flags + 9, &root->bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    GH_CUDA_TRY(cudaStreamSynchronize(st));
    // The kernels so far index only by particle and sort slot, whatever the keys hold,
    // so non-finite input is refused here, before any cell is built from it.
    if (ws.host_flags[9])
      return set_error(GH_ERR_ARG,
                       "tree: particle positions and masses must be finite (the reference's octree insert "
                       "does not terminate on NaN or infinite coordinates)");
    if (ws.host_flags[5]) return set_error(GH_ERR_TIMEOUT, "tree: radix sort look-back gave up");
    if (ws.host_flags[2] && !full_sort) {  // a long run of equal first words
      full_sort = true;
      ws.full_sort_n = n;
      continue;
    }
    if (!ws.host_flags[0]) break;
    if (ws.words >= TREE_MAX_WORDS)
      return set_error(GH_ERR_DEPTH,
                       "tree: particles share their first %d octree levels (coincident positions?)",
                       TREE_MAX_WORDS * KEY_LEVELS);
    ws.words++;
  }
  const int words = ws.words;
  const int maxdepth = ws.host_flags[1];
  const int nnodes = ws.host_flags[8];
  // 4. nodes
  GH_TRY(ensure(ws.nA, (size_t)nnodes * sizeof(WalkRec)));
  GH_TRY(ensure(ws.nC, (size_t)nnodes * sizeof(dvec4)));
  GH_TRY(ensure(ws.nM, (size_t)nnodes * sizeof(dvec4)));
  const int64_t ntiles = (n + MS_TILE - 1) / MS_TILE;
  GH_TRY(ensure(ws.fxl, (size_t)n * sizeof(FxMoments)));
  GH_TRY(ensure(ws.fxt, (size_t)(ntiles + 1) * sizeof(FxMoments)));
  // every node that is not a particle's leaf is an internal cell
  const int64_t ncells = (int64_t)nnodes - n;
  GH_TRY(ensure(ws.cells, (size_t)(ncells > 0 ? ncells : 1) * sizeof(int2)));
  NodeArrays na = node_arrays(ws);
  {
    const uint64_t* keys = (const uint64_t*)ws.keys.ptr;
    const int* lp = (const int*)ws.lp.ptr;
    const int* dep = (const int*)ws.depth.ptr;
    const int* bs = (const int*)ws.base.ptr;
    const uint32_t* perm = (const uint32_t*)ws.idx.ptr;
    int* openers = (int*)ws.flags.ptr + 4;
    FxMoments* fxl = (FxMoments*)ws.fxl.ptr;
    FxMoments* fxt = (FxMoments*)ws.fxt.ptr;
    // 5. exact prefix sums of the moments (the cells' monopoles come from them below)
    moments_scan_kernel<<<(unsigned)ntiles, MS_THREADS, 0, st>>>(pos, mass, perm, n, root, fxl, fxt);
    GH_LAUNCH_CHECK();
    moments_tiles_kernel<<<1, MS_THREADS, 0, st>>>(fxt, ntiles);
    GH_LAUNCH_CHECK();
    // 4. leaves, then the internal cells' centres, then the rest of each internal cell
    int2* cells = (int2*)ws.cells.ptr;
    nodes_kernel<<<gn, T, 0, st>>>(n, lp, dep, bs, perm, pos, mass, na, nnodes, (int*)ws.list.ptr, openers, cells,
                                   (int*)ws.flags.ptr + 6);
    GH_LAUNCH_CHECK();
    cell_centres_kernel<<<gn < 4 * 152 ? gn : 4 * 152, T, 0, st>>>(keys, words, n, lp, dep, bs, root, na,
                                                                  (const int*)ws.list.ptr, openers);
    GH_LAUNCH_CHECK();
    if (ncells > 0) {
      cells_kernel<<<(unsigned)((ncells + T - 1) / T), T, 0, st>>>(keys, words, n, lp, bs, root, na, nnodes, cells,
                                                                   (int)ncells, fxl, fxt);
      GH_LAUNCH_CHECK();
    }
  }
  out->nnodes = nnodes;
  out->maxdepth = maxdepth;
  return GH_OK;
}

// Walk counters, off unless gh_tree_stats(1): [0] warp cell steps (one 48-byte
// record read each), [1] cells visited summed over targets, [2] target-cell
// interactions, [3] exact FP64 opening tests, [4] interactions with leaves.
static bool g_stats_on = false;
static int64_t g_stats_walks = 0;
static Buffer g_stats[64];

template <bool G, bool MX, class Epi>
static void launch_walk(const NodeArrays& na, const BuiltTree& bt, const double* tpos, const uint32_t* order,
                        int64_t nt, double eps2, double theta, float lo, float hi, const Epi& epi,
                        unsigned long long* stats, cudaStream_t st) {
  const unsigned blocks = (unsigned)((nt + TW_THREADS - 1) / TW_THREADS);
  if (stats)
    tree_walk_kernel<G, MX, true, Epi><<<blocks, TW_THREADS, 0, st>>>(na.R, na.C, na.M, bt.nnodes, tpos, order, nt,
                                                                      eps2, theta, lo, hi, epi, stats);
  else
    tree_walk_kernel<G, MX, false, Epi><<<blocks, TW_THREADS, 0, st>>>(na.R, na.C, na.M, bt.nnodes, tpos, order,
                                                                       nt, eps2, theta, lo, hi, epi, nullptr);
}

template <class Epi>
static int tree_walk(TreeWS& ws, const BuiltTree& bt, const double* tpos, const uint32_t* order, int64_t nt,
                     double eps, double theta, int precision, const Epi& epi, cudaStream_t st) {
  if (nt == 0) return GH_OK;
  Trace tr("tree walk");
  const double eps2 = eps * eps;
  // theta <= 0 or NaN: the prefilter opens every cell and accepts none; below 1e-3
  // it decides nothing (every internal cell takes the exact test)
  float lo = -1.f, hi = -1.f;
  if (theta >= 1e-3) {
    lo = (float)(theta * theta * (1.0 - TREE_MARGIN));
    hi = (float)(theta * theta * (1.0 + TREE_MARGIN));
  } else if (theta > 0.0) {
    hi = INFINITY;
  }
  NodeArrays na = node_arrays(ws);
  const bool mixed = precision == GH_PREC_MIXED;
  const bool guard = mixed ? !((float)eps2 > 0.f) : eps2 == 0.0;
  unsigned long long* stats = nullptr;
  if (g_stats_on) {
    DeviceInfo di;
    GH_TRY(device_info(&di));
    Buffer& b = g_stats[di.device];
    if (!b.ptr) {
      GH_TRY(ensure(b, 8 * sizeof(unsigned long long)));
      GH_CUDA_TRY(cudaMemsetAsync(b.ptr, 0, 8 * sizeof(unsigned long long), st));
    }
    stats = (unsigned long long*)b.ptr;
    g_stats_walks++;
  }
  prof_begin(st);
  if (mixed) {
    if (guard)
      launch_walk<true, true>(na, bt, tpos, order, nt, eps2, theta, lo, hi, epi, stats, st);
    else
      launch_walk<false, true>(na, bt, tpos, order, nt, eps2, theta, lo, hi, epi, stats, st);
  } else {
    if (guard)
      launch_walk<true, false>(na, bt, tpos, order, nt, eps2, theta, lo, hi, epi, stats, st);
    else
      launch_walk<false, false>(na, bt, tpos, order, nt, eps2, theta, lo, hi, epi, stats, st);
  }
  prof_end(st);
  GH_LAUNCH_CHECK();
  return GH_OK;
}

static int check_tree_args(int64_t np, int64_t nt, double eps, int precision) {
  if (np < 0 || nt < 0) return set_error(GH_ERR_ARG, "negative particle count");
  if (precision != GH_PREC_FP64 && precision != GH_PREC_MIXED)
    return set_error(GH_ERR_ARG, "unknown precision %d", precision);
  if (!(eps >= 0.0)) return set_error(GH_ERR_ARG, "eps must be >= 0 (got %g)", eps);
  return GH_OK;
}

int tree_force(const double* pos, const double* mass, int64_t np, const double* tpos, int64_t nt, double eps,
               double theta, int precision, double* acc, cudaStream_t st) {
  GH_TRY(check_tree_args(np, nt, eps, precision));
  const bool self = (tpos == nullptr);
  if (self) nt = np;
  if (nt == 0) return GH_OK;
  if (np == 0) {
    GH_CUDA_TRY(cudaMemsetAsync(acc, 0, (size_t)nt * 3 * sizeof(double), st));
    return GH_OK;
  }
  std::lock_guard<std::recursive_mutex> lk(g_tree_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  TreeWS& ws = g_tree[di.device];
  BuiltTree bt;
  GH_TRY(tree_build(ws, pos, mass, np, eps, st, &bt, self ? nullptr : tpos, self ? 0 : nt));
  EpiStore epi{acc};
  if (self) return tree_walk(ws, bt, pos, (const uint32_t*)ws.idx.ptr, np, eps, theta, precision, epi, st);
  return tree_walk(ws, bt, tpos, bt.torder, nt, eps, theta, precision, epi, st);
}

int tree_run(double* x, double* v, const double* mass, int64_t np, int64_t nsteps, double dt, double eps,
             double theta, int precision, double* hist_x, double* hist_v, int64_t stride, cudaStream_t st) {
  GH_TRY(check_tree_args(np, 0, eps, precision));
  std::lock_guard<std::recursive_mutex> lk(g_tree_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  TreeWS& ws = g_tree[di.device];
  GH_TRY(ensure(ws.xh[0], (size_t)np * 3 * sizeof(double)));
  GH_TRY(ensure(ws.xh[1], (size_t)np * 3 * sizeof(double)));
  GH_TRY(drift_prepare_f64(x, v, np, dt, (double*)ws.xh[0].ptr, st));
  for (int64_t s = 0; s < nsteps; s++) {
    Trace step("tree dkd step");
    const int cur = (int)(s & 1), nxt = cur ^ 1;
    const double* xh = (const double*)ws.xh[cur].ptr;
    BuiltTree bt;
    GH_TRY(tree_build(ws, xh, mass, np, eps, st, &bt));
    EpiDKD epi;
    epi.x = x;
    epi.v = v;
    epi.mass = mass;
    epi.dt = dt;
    epi.src_next = nullptr;
    epi.origin = nullptr;
    epi.xh_next = (double*)ws.xh[nxt].ptr;
    epi.hist_x = epi.hist_v = nullptr;
    if (hist_x && stride > 0 && (s + 1) % stride == 0) {
      const int64_t slot = (s + 1) / stride - 1;
      epi.hist_x = hist_x + slot * np * 3;
      epi.hist_v = hist_v + slot * np * 3;
    }
    GH_TRY(tree_walk(ws, bt, xh, (const uint32_t*)ws.idx.ptr, np, eps, theta, precision, epi, st));
  }
  return GH_OK;
}

}  // namespace gh

// ---------------------------------------------------------------------------
// Invariant check of a built tree (gh_tree_validate)
// ---------------------------------------------------------------------------
// out: [0] leaves, [1] skip index out of range, [2] children that do not tile their
// cell's subtree, [3] cells with more than 8 child cells, [4] cell mass not the sum of
// its children's, [5] a child's centre of mass outside its cell, [6] walk record not
// matching the FP64 cell, [7] root subtree not the whole preorder.
namespace gh {
__global__ void tree_validate_kernel(const WalkRec* __restrict__ R, const dvec4* __restrict__ C,
                                     const dvec4* __restrict__ M, int nnodes, unsigned long long* __restrict__ out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnodes; k += gridDim.x * blockDim.x) {
    const int nx = __float_as_int(R[k].L.w);
    if (k == 0 && nx != nnodes) atomicAdd(&out[7], 1ull);
    if (nx <= k || nx > nnodes) {
      atomicAdd(&out[1], 1ull);
      continue;
    }
    const dvec4 Mk = M[k];
    if (nx == k + 1) {  // leaf: its record is its particle
      atomicAdd(&out[0], 1ull);
      const float4 A = R[k].A;
      if (A.x != (float)Mk.x || A.y != (float)Mk.y || A.z != (float)Mk.z || R[k].O.w != (float)Mk.w)
        atomicAdd(&out[6], 1ull);
      continue;
    }
    const dvec4 Ck = C[k];
    const float4 A = R[k].A;
    if (A.x != (float)Ck.x || A.y != (float)Ck.y || A.z != (float)Ck.z || A.w != (float)(Ck.w * Ck.w) ||
        R[k].O.w != (float)Mk.w)
      atomicAdd(&out[6], 1ull);
    // children: k + 1, then each one's skip index, up to this cell's skip index (at most 8
    // steps are taken; a ninth child counts as a violation)
    const double half = 0.5 * Ck.w * (1.0 + 1e-12);
    double msum = 0.0;
    int c = k + 1, kids = 0;
    while (c < nx && kids <= 8) {
      const dvec4 Mc = M[c];
      msum += Mc.w;
      if (fabs(Mc.x - Ck.x) > half || fabs(Mc.y - Ck.y) > half || fabs(Mc.z - Ck.z) > half)
        atomicAdd(&out[5], 1ull);
      const int cn = __float_as_int(R[c].L.w);
      if (cn <= c || cn > nx) break;
      c = cn;
      kids++;
    }
    if (kids > 8) atomicAdd(&out[3], 1ull);
    else if (c != nx) atomicAdd(&out[2], 1ull);
    if (!(fabs(msum - Mk.w) <= 1e-12 * fabs(Mk.w))) atomicAdd(&out[4], 1ull);
  }
}
}  // namespace gh

extern "C" int gh_tree_validate(const double* pos, const double* mass, int64_t np, double eps, int64_t* out,
                                void* stream) {
  using namespace gh;
  clear_error();
  if (!out) return set_error(GH_ERR_ARG, "tree validate: null output");
  if (np <= 0) return set_error(GH_ERR_ARG, "tree validate: no particles");
  if (!pos || !mass) return set_error(GH_ERR_ARG, "null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::recursive_mutex> lk(g_tree_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  TreeWS& ws = g_tree[di.device];
  BuiltTree bt;
  GH_TRY(tree_build(ws, pos, mass, np, eps, st, &bt));
  static Buffer counts[64];
  GH_TRY(ensure(counts[di.device], 8 * sizeof(unsigned long long)));
  unsigned long long* dc = (unsigned long long*)counts[di.device].ptr;
  GH_CUDA_TRY(cudaMemsetAsync(dc, 0, 8 * sizeof(unsigned long long), st));
  NodeArrays na = node_arrays(ws);
  tree_validate_kernel<<<2 * di.num_sms, 256, 0, st>>>(na.R, na.C, na.M, bt.nnodes, dc);
  GH_LAUNCH_CHECK();
  unsigned long long h[8];
  GH_CUDA_TRY(cudaMemcpyAsync(h, dc, sizeof(h), cudaMemcpyDeviceToHost, st));
  GH_CUDA_TRY(cudaStreamSynchronize(st));
  out[0] = bt.nnodes;
  for (int k = 0; k < 8; k++) out[k + 1] = (int64_t)h[k];
  return GH_OK;
}

extern "C" int gh_tree_stats(int enable) {
  using namespace gh;
  clear_error();
  std::lock_guard<std::recursive_mutex> lk(g_tree_mu);
  g_stats_on = enable != 0;
  return GH_OK;
}

extern "C" int gh_tree_stats_read(int64_t* out) {
  using namespace gh;
  clear_error();
  if (!out) return set_error(GH_ERR_ARG, "tree stats: null output");
  std::lock_guard<std::recursive_mutex> lk(g_tree_mu);
  DeviceInfo di;
  GH_TRY(device_info(&di));
  Buffer& b = g_stats[di.device];
  unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
  if (b.ptr) {
    GH_CUDA_TRY(cudaDeviceSynchronize());
    GH_CUDA_TRY(cudaMemcpy(h, b.ptr, sizeof(h), cudaMemcpyDeviceToHost));
    GH_CUDA_TRY(cudaMemset(b.ptr, 0, sizeof(h)));
    GH_CUDA_TRY(cudaDeviceSynchronize());
  }
  out[0] = g_stats_walks;
  for (int k = 0; k < 6; k++) out[k + 1] = (int64_t)h[k];
  g_stats_walks = 0;
  return GH_OK;
}
