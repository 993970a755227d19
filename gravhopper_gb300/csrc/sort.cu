// Stable LSD radix sort (8-bit digits, multi-word keys) and exclusive scan.
//
// Each sort pass is one launch (one-sweep, below) after one histogram launch per
// key word.  Stability inside a tile comes from giving each warp a contiguous block of
// the tile's items, ranked in order within the warp (match-any per round of 32 items,
// a warp-local running count per digit) and across warps by a prefix over the warps'
// counts; across tiles from the tiles' ticket order.
#include <chrono>
#include <mutex>

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

// ---------------------------------------------------------------------------
// One-sweep LSD passes.  The digit histograms of every pass are counted up front
// (they do not depend on the order of the keys); each pass is then one launch in
// which a CTA takes the next tile by ticket, counts its tile's digits, publishes them
// and finds its output offsets by looking back over the earlier tiles' published
// counts (decoupled look-back).  A CTA only ever waits on tiles with smaller tickets,
// which are already running, and every wait is bounded: after wait_ns nanoseconds of
// the GPU's global timer (OS_WAIT_NS in the sort; at most OS_MAX_SPINS polls either
// way) the error flag is set, the wait ends and the sort's result is garbage, but
// every write stays inside its buffers.
// ---------------------------------------------------------------------------
constexpr uint32_t OS_AGG = 1u << 30;    // status word: tile count published
constexpr uint32_t OS_INC = 2u << 30;    // status word: inclusive prefix published
constexpr uint32_t OS_VAL = (1u << 30) - 1;
constexpr int OS_MAX_SPINS = 1 << 24;
constexpr long long OS_WAIT_NS = 1000000000ll;  // one second
constexpr int OS_MAX_PASSES = 8;        // 8-bit digits of one 64-bit word
constexpr int OS_WIN = 8;               // predecessor tiles read per look-back step

__device__ __forceinline__ uint32_t ld_status(const uint32_t* p) { return *(const volatile uint32_t*)p; }
__device__ __forceinline__ void st_status(uint32_t* p, uint32_t v) { *(volatile uint32_t*)p = v; }
__device__ __forceinline__ long long global_ns() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Digit counts of every pass of one key word: out[p*256 + d].
__global__ void __launch_bounds__(RS_THREADS)
    os_hist_kernel(const uint64_t* __restrict__ kw, int64_t n, int passes, uint32_t* __restrict__ out) {
  __shared__ uint32_t h[OS_MAX_PASSES][RS_BINS];
  for (int p = 0; p < OS_MAX_PASSES; p++) h[p][threadIdx.x] = 0;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * RS_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * RS_THREADS) {
    const uint64_t k = kw[i];
    for (int p = 0; p < passes; p++) atomicAdd(&h[p][(k >> (8 * p)) & 255u], 1u);
  }
  __syncthreads();
  for (int p = 0; p < passes; p++)
    if (h[p][threadIdx.x]) atomicAdd(&out[p * RS_BINS + threadIdx.x], h[p][threadIdx.x]);
}

// Counts -> exclusive digit offsets, for `np` passes of 256 digits each, in place.
__global__ void __launch_bounds__(RS_BINS) os_offsets_kernel(uint32_t* __restrict__ off, int np) {
  __shared__ uint32_t ws[RS_BINS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < np; q++) {
    const uint32_t v = off[q * RS_BINS + threadIdx.x];
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int k = 0; k < warp; k++) before += ws[k];
    off[q * RS_BINS + threadIdx.x] = before + x - v;
    __syncthreads();
  }
}

// WK = 1 or 2: the tile's key words and payloads are loaded into registers, all
// loads issued together, before the digits are counted; WK = 0: any number of
// words, the digit word loaded first and the rest reloaded per round.
template <int WK>
__global__ void __launch_bounds__(RS_THREADS, 2)
    os_pass_kernel(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ iin, uint64_t* __restrict__ kout,
                   uint32_t* __restrict__ iout, int words, int64_t n, int w, int shift,
                   const uint32_t* __restrict__ doff, uint32_t* __restrict__ status, int* __restrict__ ticket,
                   int* __restrict__ err, long long wait_ns) {
  // Blocked layout: warp wi owns the tile's items [wi*256, wi*256+256), lane l of it
  // item wi*256 + r*32 + l in round r.  A warp ranks its items by itself (match-any per
  // round and a warp-local running count per digit); one prefix over the warps per
  // digit then gives every item its place, so the tile needs two barriers.
  constexpr int NW = RS_THREADS / 32;
  constexpr int WITEMS = 32 * RS_ROUNDS;  // items per warp
  __shared__ uint32_t warp_cnt[NW][RS_BINS];
  __shared__ uint32_t cursor[RS_BINS];
  __shared__ int s_tile;
  static_assert(RS_THREADS == RS_BINS, "one digit bin per thread");
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) s_tile = atomicAdd(ticket, 1);
#pragma unroll
  for (int k = 0; k < NW; k++) warp_cnt[k][tid] = 0;
  __syncthreads();
  const int tile = s_tile;
  const int64_t base = (int64_t)tile * RS_TILE + (int64_t)warp * WITEMS + lane;
  const uint64_t* kw = kin + (int64_t)w * n;
  unsigned dig[RS_ROUNDS];
  uint32_t rank[RS_ROUNDS];
  uint64_t kr[RS_ROUNDS][WK > 0 ? WK : 1];
  uint32_t ir[RS_ROUNDS];
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; r++) {
    const int64_t i = base + r * 32;
    if (WK > 0) {
#pragma unroll
      for (int q = 0; q < (WK > 0 ? WK : 1); q++) kr[r][q] = i < n ? kin[(int64_t)q * n + i] : 0ull;
      ir[r] = i < n ? iin[i] : 0u;
    } else {
      kr[r][0] = i < n ? kw[i] : 0ull;
    }
  }
  uint32_t* wc = warp_cnt[warp];
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; r++) {
    const int64_t i = base + r * 32;
    const uint64_t kd = (WK == 2 && w == 1) ? kr[r][WK > 1 ? 1 : 0] : kr[r][0];  // no dynamic register index
    dig[r] = i < n ? (unsigned)((kd >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, dig[r]);
    const unsigned below = __popc(peers & lanemask_lt());
    const bool valid = dig[r] < 256u;
    rank[r] = (valid ? wc[dig[r]] : 0u) + below;  // earlier rounds' count, then earlier lanes
    __syncwarp();
    if (valid && below == 0) wc[dig[r]] += (uint32_t)__popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // thread tid = digit: its count in the tile, and each warp's offset within the tile
  uint32_t cnt = 0;
#pragma unroll
  for (int k = 0; k < NW; k++) {
    const uint32_t c = warp_cnt[k][tid];
    warp_cnt[k][tid] = cnt;  // now the warp's offset for this digit
    cnt += c;
  }
  // publish this tile's count of digit tid, then add up the earlier tiles' counts
  uint32_t excl = 0;
  uint32_t* my = status + (int64_t)tile * RS_BINS + tid;
  if (tile == 0) {
    st_status(my, OS_INC | cnt);
  } else {
    st_status(my, OS_AGG | cnt);
    // look back OS_WIN tiles at a time (independent loads), nearest first
    bool done = false;
    for (int t0 = tile - 1; t0 >= 0 && !done; t0 -= OS_WIN) {
      uint32_t v[OS_WIN];
#pragma unroll
      for (int j = 0; j < OS_WIN; j++) v[j] = t0 - j >= 0 ? ld_status(status + (int64_t)(t0 - j) * RS_BINS + tid) : OS_INC;
#pragma unroll
      for (int j = 0; j < OS_WIN; j++) {
        if (done) break;
        const uint32_t* ps = status + (int64_t)(t0 - j) * RS_BINS + tid;
        if ((v[j] >> 30) == 0) {
          const long long w0 = global_ns();
          for (int spin = 0; (v[j] >> 30) == 0; spin++) {
            if (spin >= OS_MAX_SPINS || ((spin & 31) == 31 && global_ns() - w0 > wait_ns)) {
              atomicOr(err, 1);
              v[j] = OS_INC;  // give up: count the tile as empty
              break;
            }
            v[j] = ld_status(ps);
          }
        }
        excl += v[j] & OS_VAL;
        done = (v[j] & ~OS_VAL) == OS_INC;
      }
    }
    st_status(my, OS_INC | (excl + cnt));
  }
  cursor[tid] = doff[tid] + excl;
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; r++) {
    const int64_t i = base + r * 32;
    if (i < n) {
      const unsigned d = dig[r];
      const int64_t pos = (int64_t)cursor[d] + wc[d] + rank[r];
      if (WK > 0) {
#pragma unroll
        for (int q = 0; q < (WK > 0 ? WK : 1); q++) kout[(int64_t)q * n + pos] = kr[r][q];
        iout[pos] = ir[r];
      } else {
        for (int q = 0; q < words; q++) kout[(int64_t)q * n + pos] = kin[(int64_t)q * n + i];
        iout[pos] = iin[i];
      }
    }
  }
}

// Scratch layout (u32 words): digit offsets of every pass (passes * 256), tile status
// words of every pass (passes * tiles * 256), one ticket per pass, the error flag.
static int64_t os_tiles(int64_t n) { return (n + RS_TILE - 1) / RS_TILE; }

int64_t radix_scratch_words(int64_t n) {
  const int64_t passes = (int64_t)6 * OS_MAX_PASSES;  // up to six key words
  const int64_t tiles = os_tiles(n) > 0 ? os_tiles(n) : 1;
  return passes * RS_BINS + passes * tiles * RS_BINS + passes + 1;
}

int radix_sort_keys(uint64_t* keys, uint32_t* idx, uint64_t* keys_tmp, uint32_t* idx_tmp, int words,
                    int bits_per_word, int64_t n, uint32_t* scratch_u32, cudaStream_t st, int* err) {
  if (n <= 1) return GH_OK;
  if (words < 1 || words > 6) return set_error(GH_ERR_ARG, "radix sort: %d key words", words);
  const int64_t tiles = os_tiles(n);
  const int passes = (bits_per_word + 7) / 8;
  const int np = words * passes;
  uint32_t* doff = scratch_u32;
  uint32_t* status = doff + (int64_t)np * RS_BINS;
  int* tickets = (int*)(status + (int64_t)np * tiles * RS_BINS);
  int* own_err = tickets + np;
  if (!err) err = own_err;
  GH_CUDA_TRY(cudaMemsetAsync(doff, 0, sizeof(uint32_t) * ((int64_t)np * RS_BINS * (1 + tiles) + np + 1), st));
  // pass q sorts word w = words-1-q/passes on digit q%passes
  const unsigned hb = (unsigned)(tiles < 2 * 152 ? tiles : 2 * 152);
  for (int w = words - 1; w >= 0; w--) {
    os_hist_kernel<<<hb, RS_THREADS, 0, st>>>(keys + (int64_t)w * n, n, passes,
                                              doff + (int64_t)(words - 1 - w) * passes * RS_BINS);
    GH_LAUNCH_CHECK();
  }
  os_offsets_kernel<<<1, RS_BINS, 0, st>>>(doff, np);
  GH_LAUNCH_CHECK();
  uint64_t *ks = keys, *kd = keys_tmp;
  uint32_t *is = idx, *id = idx_tmp;
  for (int q = 0; q < np; q++) {
    const int w = words - 1 - q / passes, shift = 8 * (q % passes);
    const uint32_t* dq = doff + (int64_t)q * RS_BINS;
    uint32_t* sq = status + (int64_t)q * tiles * RS_BINS;
    if (words == 1)
      os_pass_kernel<1><<<(unsigned)tiles, RS_THREADS, 0, st>>>(ks, is, kd, id, words, n, w, shift, dq, sq, tickets + q,
                                                                err, OS_WAIT_NS);
    else if (words == 2)
      os_pass_kernel<2><<<(unsigned)tiles, RS_THREADS, 0, st>>>(ks, is, kd, id, words, n, w, shift, dq, sq, tickets + q,
                                                                err, OS_WAIT_NS);
    else
      os_pass_kernel<0><<<(unsigned)tiles, RS_THREADS, 0, st>>>(ks, is, kd, id, words, n, w, shift, dq, sq, tickets + q,
                                                                err, OS_WAIT_NS);
    GH_LAUNCH_CHECK();
    uint64_t* tk = ks;
    ks = kd;
    kd = tk;
    uint32_t* ti = is;
    is = id;
    id = ti;
  }
  if (ks != keys) {
    GH_CUDA_TRY(cudaMemcpyAsync(keys, ks, sizeof(uint64_t) * words * n, cudaMemcpyDeviceToDevice, st));
    GH_CUDA_TRY(cudaMemcpyAsync(idx, is, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st));
  }
  return GH_OK;
}

// ---------------------------------------------------------------------------
// Test of the bounded wait (gh_debug_sort_stall): two tiles of zero keys; the
// ticket counter starts at 1, so the only CTA takes tile 1 and looks back at tile 0,
// which nothing publishes.  Its loads and stores stay inside the two tiles' buffers:
// with the wait given up, tile 0 counts as empty and tile 1's keys go to positions
// [0, RS_TILE).
// ---------------------------------------------------------------------------
struct StallWS {
  Buffer keys, idx, scratch;
};
static StallWS g_stall[64];

int sort_stall_test(int device, long long wait_ns, cudaStream_t st, int* gave_up) {
  StallWS& ws = g_stall[device];
  const int64_t n = 2 * RS_TILE, tiles = 2;
  GH_TRY(ensure(ws.keys, 2 * n * sizeof(uint64_t)));
  GH_TRY(ensure(ws.idx, 2 * n * sizeof(uint32_t)));
  // digit offsets (256), tile status words (2 x 256), ticket, error flag
  GH_TRY(ensure(ws.scratch, (RS_BINS * (1 + tiles) + 2) * sizeof(uint32_t)));
  uint64_t* kin = (uint64_t*)ws.keys.ptr;
  uint32_t* iin = (uint32_t*)ws.idx.ptr;
  uint32_t* doff = (uint32_t*)ws.scratch.ptr;
  uint32_t* status = doff + RS_BINS;
  int* ticket = (int*)(status + tiles * RS_BINS);
  int* err = ticket + 1;
  GH_CUDA_TRY(cudaMemsetAsync(ws.keys.ptr, 0, ws.keys.bytes, st));
  GH_CUDA_TRY(cudaMemsetAsync(ws.idx.ptr, 0, ws.idx.bytes, st));
  GH_CUDA_TRY(cudaMemsetAsync(ws.scratch.ptr, 0, (RS_BINS * (1 + tiles) + 2) * sizeof(uint32_t), st));
  GH_CUDA_TRY(cudaMemsetAsync(ticket, 1, 1, st));  // ticket = 1 (little-endian low byte)
  os_hist_kernel<<<1, RS_THREADS, 0, st>>>(kin, n, 1, doff);
  GH_LAUNCH_CHECK();
  os_offsets_kernel<<<1, RS_BINS, 0, st>>>(doff, 1);
  GH_LAUNCH_CHECK();
  os_pass_kernel<1><<<1, RS_THREADS, 0, st>>>(kin, iin, kin + n, iin + n, 1, n, 0, 0, doff, status, ticket, err,
                                              wait_ns);
  GH_LAUNCH_CHECK();
  int h = 0;
  GH_CUDA_TRY(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  GH_CUDA_TRY(cudaStreamSynchronize(st));
  *gave_up = h;
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

extern "C" int gh_debug_sort_stall(int64_t wait_ns, int64_t* waited_ns) {
  using namespace gh;
  clear_error();
  if (wait_ns < 0 || wait_ns > 10000000000ll) return set_error(GH_ERR_ARG, "wait_ns must be in [0, 1e10]");
  DeviceInfo di;
  GH_TRY(device_info(&di));
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  const auto t0 = std::chrono::steady_clock::now();
  int gave_up = 0;
  GH_TRY(sort_stall_test(di.device, (long long)wait_ns, nullptr, &gave_up));
  if (waited_ns)
    *waited_ns = (int64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0)
                     .count();
  if (gave_up) return set_error(GH_ERR_TIMEOUT, "radix sort look-back gave up after %lld ns", (long long)wait_ns);
  return GH_OK;
}
