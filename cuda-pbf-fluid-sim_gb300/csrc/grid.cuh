// grid.cuh - cell keys, cell tables and compaction (host launch helpers).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pbf/parameters.h"

namespace pbf {

// KHash in the reference layout (sim/hash_keys.cu:14-27).
cudaError_t launch_hash_keys_ref(uint32_t* keys, uint32_t* indices, const float4* pos, const sim::GridBounds& g,
                                 uint32_t N, cudaStream_t s);

// Reference dense table (sim/cell_ranges.cu): start = 0xFFFFFFFF / end = 0
// for empty cells; every cell written.
cudaError_t launch_cell_ranges_ref(uint32_t* start, uint32_t* end, const uint32_t* keys_sorted, uint32_t N,
                                   uint32_t numCells, cudaStream_t s);

// Dense lower-bound table: lb[c] = first sorted slot with key >= c, for
// c in [0, numCells] (numCells + 1 entries).
cudaError_t launch_cell_lb(uint32_t* lb, const uint32_t* keys_sorted, uint32_t N, uint32_t numCells,
                           cudaStream_t s);

// Reference dense table materialised from a lower-bound table.
cudaError_t launch_lb_to_ranges(uint32_t* start, uint32_t* end, const uint32_t* lb, uint32_t numCells,
                                cudaStream_t s);

// Compaction tiles: kCompactThreads threads, kCompactItems sorted keys each
// (one look-back status word per tile in the scratch).
constexpr int kCompactThreads = 256;
constexpr int kCompactItems = 16;
constexpr int kCompactTile = kCompactThreads * kCompactItems;  // 4096 slots

// Compact table (sim/cell_compact.cu): unique keys, segment offsets,
// terminator and count, in one pass with decoupled look-back.  seg (may be
// null) receives the segment index of every sorted slot.
size_t compact_scratch_bytes(uint32_t N);
cudaError_t launch_compact(void* d_scratch, size_t scratch_bytes, uint32_t* unique_keys, uint32_t* offsets,
                           uint32_t* count, uint32_t* seg, const uint32_t* keys_sorted, uint32_t N, cudaStream_t s,
                           uint32_t* err);

// Device powf (fn 0), sqrtf (fn 1), division (fn 2) and the fast mode's
// compensated x^4 (fn 3) on arrays.
cudaError_t eval_math(int fn, const float* a, const float* b, float* out, uint32_t n, cudaStream_t s);

// Exhaustive check of the s_corr exponent's n = 4 form (see
// pbf_selftest_powf4); n_runtime must be 4.
cudaError_t selftest_powf4(float n_runtime, unsigned long long* d_mismatches, uint32_t* d_first, cudaStream_t s);

// Bounded-wait self-test (see pbf_selftest_bounded_wait).
cudaError_t selftest_bounded_wait(uint32_t spin_limit, uint32_t* d_scratch4, cudaStream_t s);

}  // namespace pbf
