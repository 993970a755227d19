// Stable LSD radix sort of multi-word 64-bit keys with a 32-bit payload, and an
// exclusive scan of int32 arrays.  Used by the octree build.
#pragma once

#include "gh_common.cuh"

namespace gh {

constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 8;                       // items per thread per tile
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;    // 2048 keys per block
constexpr int RS_BINS = 256;                       // 8-bit digits

// Sorts `n` keys of `words` 64-bit words each (word 0 most significant; arrays are
// word-major: key word w of item i at keys[w*n + i]) together with `idx`, stably.
// Only the low `bits_per_word` bits of each word are examined.  `keys_tmp`/`idx_tmp`
// are scratch of the same sizes.  On return the sorted data is in keys/idx.
// `scratch_u32` must hold radix_scratch_words(n) entries.  At most 6 words.  A
// bounded wait that gave up sets *err (device int; NULL: a flag in the scratch) and
// leaves the result undefined.
int64_t radix_scratch_words(int64_t n);
int radix_sort_keys(uint64_t* keys, uint32_t* idx, uint64_t* keys_tmp, uint32_t* idx_tmp, int words,
                    int bits_per_word, int64_t n, uint32_t* scratch_u32, cudaStream_t st, int* err = nullptr);

// Runs one sort pass whose look-back waits on a tile that is never published (see
// sort.cu); *gave_up receives the error flag the bounded wait set.
int sort_stall_test(int device, long long wait_ns, cudaStream_t st, int* gave_up);

// Exclusive scan of in[0..n) into out[0..n] (out[n] = total).  `scratch` must hold
// scan_scratch_ints(n) entries.  out may alias in.
int64_t scan_scratch_ints(int64_t n);
int exclusive_scan_i32(const int* in, int* out, int64_t n, int* scratch, cudaStream_t st);

}  // namespace gh
