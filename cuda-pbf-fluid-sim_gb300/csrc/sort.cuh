// sort.cuh - onesweep LSD radix sort of (uint32 key, uint32 value) pairs.
//
// Replaces cub::DeviceRadixSort::SortPairs as called by the reference
// (sim/sort_pairs.cu:11,23): stable, ascending, key bits [0, num_bits).
//
//   1. k_sort_hist   one read of the keys: 256-bin digit histograms of every
//                    pass at once; the last block scans them into global
//                    digit offsets and marks passes whose digit is constant
//                    (skipped: a stable sort by a constant digit is the
//                    identity).
//   2. k_sort_pass   one launch per 8-bit digit: each block takes the next
//                    tile id (atomic ticket), ranks its keys stably with
//                    __match_any_sync warp multisplit, publishes its digit
//                    counts and resolves its global offsets by decoupled
//                    look-back over the previous tiles (bounded spins), then
//                    scatters.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace pbf {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
// Keys per thread of a pass: large sorts take 30 (7,680 per tile, so that a
// 1M-key pass is one wave of 137 tiles with short look-back chains), small
// ones 15 (more, shorter tiles: at 65,536 keys 18 tiles instead of 9).
constexpr int kSortItemsSmall = 15;
constexpr int kSortItemsLarge = 30;
constexpr uint32_t kSortLargeFrom = 1u << 19;  // keys
inline int sort_items_for(uint32_t N) { return N >= kSortLargeFrom ? kSortItemsLarge : kSortItemsSmall; }
constexpr int kSortMaxPasses = 4;

struct SortInfo {
    uint32_t hist[kSortMaxPasses][256];
    uint32_t offs[kSortMaxPasses][256];
    uint32_t active[kSortMaxPasses];
    uint32_t src[kSortMaxPasses];
    uint32_t dst[kSortMaxPasses];
    uint32_t tileCounter[kSortMaxPasses];
    uint32_t done;
    uint32_t nactive;
    uint32_t err;
    uint32_t pad;
};

// Bytes of temporary storage for N pairs over num_bits key bits.
size_t sort_temp_bytes(uint32_t N, int num_bits);

// Sorts (keys_in, vals_in) into (keys_out, vals_out).  vals_in == nullptr
// means vals_in[i] = i.  keys_in/vals_in are not modified.  err (device
// pointer, may be null) receives kErr* bits of bounded waits that gave up;
// when null, the SortInfo inside d_temp holds them.
cudaError_t sort_pairs(void* d_temp, size_t temp_bytes, const uint32_t* keys_in, uint32_t* keys_out,
                       const uint32_t* vals_in, uint32_t* vals_out, uint32_t N, int num_bits, cudaStream_t s,
                       uint32_t* err);

// Number of key bits needed to hold values in [0, max_key].
inline int bits_for(uint32_t max_key) {
    int b = 0;
    while (b < 32 && (max_key >> b) != 0u) ++b;
    return b == 0 ? 1 : b;
}

}  // namespace pbf
