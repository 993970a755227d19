// Stable LSD radix sort (8-bit digits, multi-word keys) and exclusive scan.
//
// Each sort pass is three launches: per-tile digit histograms, one exclusive scan
// of the digit-major histogram table (giving every tile its output offset per
// digit), and a stable scatter.  Stability inside a tile comes from processing the
// tile in rounds of one item per thread (item order = round, then thread) and
// ranking equal digits within a warp with __match_any_sync, across warps with a
// per-round prefix over the warp counts.
#include "sort.cuh"

namespace gh {

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Exclusive scan over a 1024-thread block of one value per thread; returns the
// thread's exclusive prefix and writes the block total to *total.
__device__ __forceinline__ int64_t block_exclusive_scan_1024(int64_t v, int64_t* total) {
  __shared__ int64_t warp_sums[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t s = warp_sums[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    warp_sums[lane] = s;
  }
  __syncthreads();
  int64_t pre = (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
  *total = warp_sums[31];
  __syncthreads();
  return pre;
}

__global__ void __launch_bounds__(RS_THREADS)
    rs_hist_kernel(const uint64_t* __restrict__ kw, int64_t n, int shift, uint32_t* __restrict__ hist,
                   int nb) {
  __shared__ uint32_t cnt[RS_BINS];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; r++) {
    int64_t i = base + r * RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(kw[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * nb + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(RS_THREADS)
    rs_scatter_kernel(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ iin,
                      uint64_t* __restrict__ kout, uint32_t* __restrict__ iout, int words, int64_t n,
                      int w, int shift, const uint32_t* __restrict__ hist, int nb) {
  constexpr int NW = RS_THREADS / 32;
  __shared__ uint32_t warp_cnt[NW][RS_BINS];
  __shared__ uint32_t warp_off[NW][RS_BINS];
  __shared__ uint32_t cursor[RS_BINS];
  __shared__ uint32_t round_tot[RS_BINS];
  static_assert(RS_THREADS == RS_BINS, "one digit bin per thread");
  const int tid = threadIdx.x, warp = tid >> 5;
#pragma unroll
  for (int k = 0; k < NW; k++) warp_cnt[k][tid] = 0;
  cursor[tid] = hist[(int64_t)tid * nb + blockIdx.x];
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  const uint64_t* kw = kin + (int64_t)w * n;
  for (int r = 0; r < RS_ROUNDS; r++) {
    const int64_t i = base + r * RS_THREADS + tid;
    const bool valid = i < n;
    const unsigned d = valid ? (unsigned)((kw[i] >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned rank = __popc(peers & lanemask_lt());
    if (valid && rank == 0) warp_cnt[warp][d] = __popc(peers);
    __syncthreads();
    {
      uint32_t run = 0;
#pragma unroll
      for (int k = 0; k < NW; k++) {
        uint32_t c = warp_cnt[k][tid];
        warp_off[k][tid] = run;
        run += c;
        warp_cnt[k][tid] = 0;
      }
      round_tot[tid] = run;
    }
    __syncthreads();
    if (valid) {
      const int64_t pos = (int64_t)cursor[d] + warp_off[warp][d] + rank;
      for (int q = 0; q < words; q++) kout[(int64_t)q * n + pos] = kin[(int64_t)q * n + i];
      iout[pos] = iin[i];
    }
    __syncthreads();
    cursor[tid] += round_tot[tid];
    __syncthreads();
  }
}

// Scratch layout: the digit-major histogram table (RS_BINS * nb + 1 entries, scanned
// in place) followed by the multi-block scan's tile sums.
int64_t radix_scratch_words(int64_t n) {
  const int64_t nb = (n + RS_TILE - 1) / RS_TILE;
  const int64_t m = (int64_t)RS_BINS * (nb > 0 ? nb : 1);
  return m + 1 + scan_scratch_ints(m);
}

int radix_sort_keys(uint64_t* keys, uint32_t* idx, uint64_t* keys_tmp, uint32_t* idx_tmp, int words,
                    int bits_per_word, int64_t n, uint32_t* scratch_u32, cudaStream_t st) {
  if (n <= 1) return GH_OK;
  const int nb = (int)((n + RS_TILE - 1) / RS_TILE);
  const int passes = (bits_per_word + 7) / 8;
  uint64_t *ks = keys, *kd = keys_tmp;
  uint32_t *is = idx, *id = idx_tmp;
  for (int w = words - 1; w >= 0; w--) {
    for (int p = 0; p < passes; p++) {
      const int shift = 8 * p;
      rs_hist_kernel<<<nb, RS_THREADS, 0, st>>>(ks + (int64_t)w * n, n, shift, scratch_u32, nb);
      GH_LAUNCH_CHECK();
      {
        const int64_t m = (int64_t)RS_BINS * nb;
        int* table = (int*)scratch_u32;
        GH_TRY(exclusive_scan_i32(table, table, m, table + m + 1, st));
      }
      rs_scatter_kernel<<<nb, RS_THREADS, 0, st>>>(ks, is, kd, id, words, n, w, shift, scratch_u32, nb);
      GH_LAUNCH_CHECK();
      uint64_t* tk = ks;
      ks = kd;
      kd = tk;
      uint32_t* ti = is;
      is = id;
      id = ti;
    }
  }
  if (ks != keys) {
    GH_CUDA_TRY(cudaMemcpyAsync(keys, ks, sizeof(uint64_t) * words * n, cudaMemcpyDeviceToDevice, st));
    GH_CUDA_TRY(cudaMemcpyAsync(idx, is, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st));
  }
  return GH_OK;
}

// ---------------------------------------------------------------------------
// Exclusive scan of int32 (three phases).
// ---------------------------------------------------------------------------
constexpr int SC_THREADS = 1024;
constexpr int SC_ITEMS = 4;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

__global__ void __launch_bounds__(SC_THREADS)
    scan_tile_kernel(const int* __restrict__ in, int* __restrict__ out, int64_t n, int* __restrict__ sums) {
  const int64_t b0 = (int64_t)blockIdx.x * SC_TILE + (int64_t)threadIdx.x * SC_ITEMS;
  int v[SC_ITEMS];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < SC_ITEMS; k++) {
    v[k] = (b0 + k < n) ? in[b0 + k] : 0;
    s += v[k];
  }
  int64_t total;
  int64_t pre = block_exclusive_scan_1024(s, &total);
#pragma unroll
  for (int k = 0; k < SC_ITEMS; k++) {
    if (b0 + k < n) out[b0 + k] = (int)pre;
    pre += v[k];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = (int)total;
}

// Exclusive scan of the tile sums (nb entries) in place, sums[nb] = grand total.
__global__ void __launch_bounds__(SC_THREADS) scan_sums_kernel(int* __restrict__ sums, int64_t nb) {
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t c0 = 0; c0 < nb; c0 += SC_THREADS) {
    int64_t i = c0 + threadIdx.x;
    int64_t v = i < nb ? sums[i] : 0;
    int64_t total;
    int64_t pre = block_exclusive_scan_1024(v, &total);
    if (i < nb) sums[i] = (int)(carry + pre);
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[nb] = (int)carry;
}

__global__ void scan_add_kernel(int* __restrict__ out, int64_t n, const int* __restrict__ sums, int64_t nb) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / SC_TILE];
  if (i == 0) out[n] = sums[nb];
}

int64_t scan_scratch_ints(int64_t n) { return (n + SC_TILE - 1) / SC_TILE + 2; }

int exclusive_scan_i32(const int* in, int* out, int64_t n, int* scratch, cudaStream_t st) {
  if (n == 0) {
    GH_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int), st));
    return GH_OK;
  }
  const int64_t nb = (n + SC_TILE - 1) / SC_TILE;
  scan_tile_kernel<<<(unsigned)nb, SC_THREADS, 0, st>>>(in, out, n, scratch);
  GH_LAUNCH_CHECK();
  scan_sums_kernel<<<1, SC_THREADS, 0, st>>>(scratch, nb);
  GH_LAUNCH_CHECK();
  scan_add_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, scratch, nb);
  GH_LAUNCH_CHECK();
  return GH_OK;
}

}  // namespace gh
