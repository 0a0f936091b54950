// grid.cu - cell keys, dense tables and single-pass compaction.
#include "grid.cuh"

#include "pbf_common.cuh"

namespace pbf {
namespace {

__global__ void k_hash_keys_ref(uint32_t* __restrict__ keys, uint32_t* __restrict__ indices,
                                const float4* __restrict__ pos, sim::GridBounds g, uint32_t N) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    keys[i] = cell_key(pos[i], g);
    indices[i] = i;
}

__device__ __forceinline__ uint32_t lower_bound_keys(const uint32_t* __restrict__ keys, uint32_t N, uint32_t c) {
    uint32_t lo = 0, hi = N;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(keys + mid) < c) lo = mid + 1; else hi = mid;
    }
    return lo;
}

constexpr uint32_t kCellsPerThread = 8;
constexpr uint32_t kLbUnset = 0xFFFFFFFFu;

// lb[c] = first sorted slot whose key is >= c, c = 0 .. numCells, in two
// passes over a table preset to kLbUnset.  Pass one, a thread per slot,
// writes the cells that have particles: lb[k] = p at the first slot p of key
// k, and lb[numCells] at the first slot past the grid (N when every key is
// inside it).
__global__ void k_cell_lb_mark(uint32_t* __restrict__ lb, const uint32_t* __restrict__ keys, uint32_t N,
                               uint32_t numCells) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    const uint32_t k = keys[p];
    const uint32_t kp = p > 0 ? keys[p - 1] : 0u;
    if (k < numCells) {
        if (p == 0 || kp != k) lb[k] = p;
        if (p == N - 1) lb[numCells] = N;
    } else if (p == 0 || kp < numCells) {
        lb[numCells] = p;
    }
}

// Pass two, a warp per block of 32 windows of 32 consecutive cells: an empty
// cell takes the value of the next cell with particles (no key lies between
// them).  The warp first finds each window's first marked value (lane j holds
// window j's), then each window's carry, the first marked value of a later
// window in the block, with a reverse shuffle scan; only a block whose tail
// has no marked cell searches the keys, once, for the first cell after it.
// Inside a window an empty cell takes the next marked lane's value by shuffle.
// Cells past the table count as marked with N, which only matters when N = 0.
constexpr uint32_t kLbBlockCells = 1024;
__global__ void k_cell_lb_fill(uint32_t* __restrict__ lb, const uint32_t* __restrict__ keys, uint32_t N,
                               uint32_t numCells) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t warp = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t base = warp * kLbBlockCells;
    if (base > numCells) return;  // warp-uniform
    // window firsts: lane j <- first marked value of window j (kLbUnset if none)
    uint32_t first = kLbUnset;
#pragma unroll 4
    for (uint32_t j = 0; j < 32u; ++j) {
        const uint64_t c = base + 32u * j + lane;
        const uint32_t v = c <= numCells ? lb[c] : N;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, v != kLbUnset);
        const uint32_t f = __shfl_sync(0xFFFFFFFFu, v, m ? int(__ffs(m)) - 1 : 0);
        if (lane == j) first = m ? f : kLbUnset;
    }
    // carry of window j: the first marked value of windows j + 1 .. 31, or past the block
    uint32_t later = __shfl_down_sync(0xFFFFFFFFu, first, 1);
    if (lane == 31u) later = kLbUnset;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_down_sync(0xFFFFFFFFu, later, o);
        if (later == kLbUnset && lane + uint32_t(o) < 32u) later = t;
    }
    if (__any_sync(0xFFFFFFFFu, later == kLbUnset)) {
        // first cell after the block (<= numCells wherever a lane needs it)
        uint32_t past = 0;
        if (lane == 0) past = base + kLbBlockCells <= numCells ? lower_bound_keys(keys, N, uint32_t(base + kLbBlockCells)) : N;
        past = __shfl_sync(0xFFFFFFFFu, past, 0);
        if (later == kLbUnset) later = past;
    }
    // fill
#pragma unroll 4
    for (uint32_t j = 0; j < 32u; ++j) {
        const uint64_t c = base + 32u * j + lane;
        const uint32_t v = c <= numCells ? lb[c] : N;
        const uint32_t marked = __ballot_sync(0xFFFFFFFFu, v != kLbUnset);
        const uint32_t after = marked & (0xFFFFFFFFu << lane);  // marked lanes at or after this one
        const uint32_t next = __shfl_sync(0xFFFFFFFFu, v, after ? int(__ffs(after)) - 1 : 0);
        const uint32_t carry = __shfl_sync(0xFFFFFFFFu, later, int(j));
        if (c <= numCells && v == kLbUnset) lb[c] = after ? next : carry;
    }
}

__global__ void k_cell_ranges_ref(uint32_t* __restrict__ start, uint32_t* __restrict__ end,
                                  const uint32_t* __restrict__ keys, uint32_t N, uint32_t numCells) {
    const uint64_t c0 = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) * kCellsPerThread;
    if (c0 >= numCells) return;
    uint32_t p = lower_bound_keys(keys, N, uint32_t(c0));
    const uint64_t c1 = min(c0 + kCellsPerThread, uint64_t(numCells));
    for (uint64_t c = c0; c < c1; ++c) {
        while (p < N && __ldg(keys + p) < uint32_t(c)) ++p;
        const uint32_t b = p;
        while (p < N && __ldg(keys + p) == uint32_t(c)) ++p;
        start[c] = (p > b) ? b : 0xFFFFFFFFu;
        end[c] = (p > b) ? p : 0u;
    }
}

__global__ void k_lb_to_ranges(uint32_t* __restrict__ start, uint32_t* __restrict__ end,
                               const uint32_t* __restrict__ lb, uint32_t numCells) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= numCells) return;
    const uint32_t b = lb[c], e = lb[c + 1];
    start[c] = (e > b) ? b : 0xFFFFFFFFu;
    end[c] = (e > b) ? e : 0u;
}

// ------------------------------------------------------------ compaction

// Values of the compaction's count word besides a count (<= N < 2^30).
constexpr uint32_t kCountPending = 0xFEFEFEFEu;  // a byte-wise memset value
constexpr uint32_t kCountInvalid = 0xFFFFFFFFu;

struct CompactInfo {
    uint32_t tileCounter;
    uint32_t pad[63];
};

size_t compact_layout_status_off() { return 256; }

// Segment starts: within a warp row (32 consecutive sorted slots) the lanes
// holding equal keys are grouped with __match_any_sync; the lowest lane of a
// group starts a segment unless it is lane 0 and the previous slot (in the
// previous row) carries the same key.  Tile counts are combined with a
// decoupled look-back, so the whole table is built in one launch.
__global__ void __launch_bounds__(kCompactThreads) k_compact(const uint32_t* __restrict__ keys, uint32_t N,
                                                             uint32_t* __restrict__ uk, uint32_t* __restrict__ off,
                                                             uint32_t* __restrict__ count, uint32_t* __restrict__ seg,
                                                             CompactInfo* info, uint32_t* status, uint32_t numTiles,
                                                             uint32_t* err) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[kCompactThreads / 32];
    __shared__ uint32_t s_excl;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) s_tile = atomicAdd(&info->tileCounter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * uint32_t(kCompactTile) + uint32_t(warp) * (32u * kCompactItems) + uint32_t(lane);
    uint32_t key[kCompactItems];
    uint32_t rowBefore[kCompactItems];  // flags in this warp before row j
    uint32_t ballots[kCompactItems];
    uint32_t wcount = 0;
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int j = 0; j < kCompactItems; ++j) {
        const uint32_t idx = base + uint32_t(j) * 32u;
        const bool valid = idx < N;
        key[j] = valid ? keys[idx] : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key[j]);
        const bool first = (__ffs(peers) - 1) == lane;
        bool flag = valid && first;
        if (flag && lane == 0 && idx > 0) flag = keys[idx - 1] != key[j];
        ballots[j] = __ballot_sync(0xFFFFFFFFu, flag);
        rowBefore[j] = wcount;
        wcount += __popc(ballots[j]);
    }
    if (lane == 0) s_warp[warp] = wcount;
    __syncthreads();
    if (t == 0) {
        uint32_t run = 0;
        for (int w = 0; w < kCompactThreads / 32; ++w) {
            const uint32_t c = s_warp[w];
            s_warp[w] = run;
            run += c;
        }
        uint32_t* st = status + tile;
        uint32_t excl = 0;
        bool gave_up = false;
        if (tile == 0) {
            st_relaxed(st, kFlagPrefix | run);
        } else {
            st_relaxed(st, kFlagAggregate | run);
            excl = lookback_exclusive(status, tile, 1u, err, kSpinLimit, &gave_up);
            st_relaxed(st, kFlagPrefix | ((excl + run) & kCountMask));
        }
        s_excl = excl;
        // The count starts as kCountPending (set before the launch).  A tile
        // whose look-back gave up marks the table invalid with 0xFFFFFFFF; the
        // last tile's count only replaces the pending value, so the mark
        // survives in either order.  (excl can only fall short of the true
        // prefix, so every index written stays below N.)
        if (gave_up) atomicExch(count, kCountInvalid);
        if (tile == numTiles - 1u) {
            const uint32_t M = excl + run;
            off[M] = N;
            if (!gave_up) atomicCAS(count, kCountPending, M);
        }
    }
    __syncthreads();
    const uint32_t wbase = s_excl + s_warp[warp];
#pragma unroll
    for (int j = 0; j < kCompactItems; ++j) {
        const uint32_t idx = base + uint32_t(j) * 32u;
        if (idx >= N) break;
        const uint32_t b = ballots[j];
        const uint32_t before = wbase + rowBefore[j] + __popc(b & lt);  // flags strictly before idx
        if ((b >> lane) & 1u) {
            uk[before] = key[j];
            off[before] = idx;
            if (seg) seg[idx] = before;
        } else if (seg) {
            seg[idx] = before - 1u;
        }
    }
}

// Self-test of the bounded wait: tile 1 looks back at tile 0, whose status
// nobody publishes; the poll loop must give up after spin_limit polls, set
// the error bit and return.
__global__ void k_selftest_lookback(const uint32_t* status, uint32_t spin_limit, uint32_t* err, uint32_t* out) {
    const uint32_t v = lookback_exclusive(status, 1u, 1u, err, spin_limit);
    if (threadIdx.x == 0) *out = v;
}

// Device math used by the neighbour kernels, evaluated on arrays (for
// checking CPU restatements against the GPU's results).
__global__ void k_eval_math(int fn, const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ out,
                            uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float r;
    switch (fn) {
        case 0: r = powf(a[i], b[i]); break;
        case 1: r = sqrtf(a[i]); break;
        case 2: r = a[i] / b[i]; break;
        case 3: r = pow4_compensated(a[i]); break;
        default: r = 0.f; break;
    }
    out[i] = r;
}

// scorr_pow(x, 4) against powf(x, n) with n = 4 known only at run time, on
// every non-negative float bit pattern up to +inf, 16 per thread.
__global__ void k_selftest_powf4(float n, unsigned long long* __restrict__ mismatches, uint32_t* __restrict__ first) {
    const uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) * 16u;
    unsigned long long local = 0;
    for (uint32_t u = 0; u < 16u; ++u) {
        const uint32_t bits = base + u;
        if (bits > 0x7F800000u) break;
        const float x = __uint_as_float(bits);
        if (__float_as_uint(scorr_pow(x, 4.0f)) != __float_as_uint(powf(x, n))) {
            ++local;
            atomicMin(first, bits);
        }
    }
    if (local) atomicAdd(mismatches, local);
}

}  // namespace

cudaError_t selftest_powf4(float n_runtime, unsigned long long* d_mismatches, uint32_t* d_first, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(d_mismatches, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_first, 0xFF, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const uint32_t threads = 0x7F800000u / 16u + 1u;
    k_selftest_powf4<<<blocks_for(threads, 256), 256, 0, s>>>(n_runtime, d_mismatches, d_first);
    return cudaGetLastError();
}

cudaError_t eval_math(int fn, const float* a, const float* b, float* out, uint32_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_eval_math<<<blocks_for(n, 256), 256, 0, s>>>(fn, a, b, out, n);
    return cudaGetLastError();
}

cudaError_t selftest_bounded_wait(uint32_t spin_limit, uint32_t* d_scratch4, cudaStream_t s) {
    // d_scratch4: [0] status of tile 0 (kept 0 = never published), [1] err, [2] out
    cudaError_t e = cudaMemsetAsync(d_scratch4, 0, 4 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    k_selftest_lookback<<<1, 32, 0, s>>>(d_scratch4, spin_limit, d_scratch4 + 1, d_scratch4 + 2);
    return cudaGetLastError();
}

cudaError_t launch_hash_keys_ref(uint32_t* keys, uint32_t* indices, const float4* pos, const sim::GridBounds& g,
                                 uint32_t N, cudaStream_t s) {
    if (N == 0) return cudaSuccess;
    k_hash_keys_ref<<<blocks_for(N, 256), 256, 0, s>>>(keys, indices, pos, g, N);
    return cudaGetLastError();
}

cudaError_t launch_cell_ranges_ref(uint32_t* start, uint32_t* end, const uint32_t* keys_sorted, uint32_t N,
                                   uint32_t numCells, cudaStream_t s) {
    if (numCells == 0) return cudaSuccess;
    const uint64_t threads = (uint64_t(numCells) + kCellsPerThread - 1) / kCellsPerThread;
    k_cell_ranges_ref<<<blocks_for(threads, 256), 256, 0, s>>>(start, end, keys_sorted, N, numCells);
    return cudaGetLastError();
}

cudaError_t launch_cell_lb(uint32_t* lb, const uint32_t* keys_sorted, uint32_t N, uint32_t numCells,
                           cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(lb, 0xFF, (size_t(numCells) + 1u) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    if (N > 0) k_cell_lb_mark<<<blocks_for(N, 256), 256, 0, s>>>(lb, keys_sorted, N, numCells);
    const uint64_t warps = (uint64_t(numCells) + kLbBlockCells) / kLbBlockCells;  // numCells + 1 cells
    k_cell_lb_fill<<<blocks_for(warps * 32u, 256), 256, 0, s>>>(lb, keys_sorted, N, numCells);
    return cudaGetLastError();
}

cudaError_t launch_lb_to_ranges(uint32_t* start, uint32_t* end, const uint32_t* lb, uint32_t numCells,
                                cudaStream_t s) {
    if (numCells == 0) return cudaSuccess;
    k_lb_to_ranges<<<blocks_for(numCells, 256), 256, 0, s>>>(start, end, lb, numCells);
    return cudaGetLastError();
}

size_t compact_scratch_bytes(uint32_t N) {
    const uint32_t tiles = N == 0 ? 1u : (N + kCompactTile - 1) / kCompactTile;
    return compact_layout_status_off() + ((size_t(tiles) * 4u + 255u) & ~size_t(255));
}

cudaError_t launch_compact(void* d_scratch, size_t scratch_bytes, uint32_t* unique_keys, uint32_t* offsets,
                           uint32_t* count, uint32_t* seg, const uint32_t* keys_sorted, uint32_t N, cudaStream_t s,
                           uint32_t* err) {
    if (N == 0) {
        // sim/cell_compact.cu:189-193: offsets[0] = 0, count = 0.
        cudaError_t e = cudaMemsetAsync(offsets, 0, sizeof(uint32_t), s);
        if (e != cudaSuccess) return e;
        return cudaMemsetAsync(count, 0, sizeof(uint32_t), s);
    }
    if (!d_scratch || scratch_bytes < compact_scratch_bytes(N)) return cudaErrorInvalidValue;
    const uint32_t tiles = (N + kCompactTile - 1) / kCompactTile;
    char* base = static_cast<char*>(d_scratch);
    CompactInfo* info = reinterpret_cast<CompactInfo*>(base);
    uint32_t* status = reinterpret_cast<uint32_t*>(base + compact_layout_status_off());
    if (!err) err = &info->pad[0];
    cudaError_t e = cudaMemsetAsync(base, 0, compact_layout_status_off() + size_t(tiles) * 4u, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(count, 0xFE, sizeof(uint32_t), s);  // kCountPending
    if (e != cudaSuccess) return e;
    k_compact<<<tiles, kCompactThreads, 0, s>>>(keys_sorted, N, unique_keys, offsets, count, seg, info, status, tiles,
                                                err);
    return cudaGetLastError();
}

}  // namespace pbf
