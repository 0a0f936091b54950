// sort.cu - onesweep LSD radix sort (see sort.cuh).
#include "sort.cuh"

#include "pbf_common.cuh"

namespace pbf {
namespace {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

struct SortLayout {
    int passes;
    uint32_t tiles;
    size_t info_off, status_off, keys_alt_off, vals_alt_off, total, zero_bytes;
};

SortLayout layout_for(uint32_t N, int num_bits) {
    SortLayout L{};
    L.passes = (num_bits + 7) / 8;
    if (L.passes < 1) L.passes = 1;
    if (L.passes > kSortMaxPasses) L.passes = kSortMaxPasses;
    const uint32_t tile = uint32_t(kSortThreads * sort_items_for(N));
    L.tiles = (N + tile - 1) / tile;
    if (L.tiles == 0) L.tiles = 1;
    L.info_off = 0;
    L.status_off = align_up(sizeof(SortInfo));
    const size_t status_bytes = size_t(L.passes) * L.tiles * 256u * sizeof(uint32_t);
    L.keys_alt_off = align_up(L.status_off + status_bytes);
    L.vals_alt_off = align_up(L.keys_alt_off + size_t(N) * 4u);
    L.total = align_up(L.vals_alt_off + size_t(N) * 4u);
    L.zero_bytes = L.status_off + status_bytes;
    return L;
}

struct SortBufs {
    const uint32_t* keys_in;
    const uint32_t* vals_in;  // null: identity
    uint32_t* keys_alt;
    uint32_t* vals_alt;
    uint32_t* keys_out;
    uint32_t* vals_out;
};

__device__ __forceinline__ uint32_t digit_of(uint32_t key, int begin_bit, int end_bit, int pass) {
    const int shift = begin_bit + pass * 8;
    const int nb = min(8, end_bit - shift);
    return (key >> shift) & ((1u << nb) - 1u);
}

// Upfront histogram of every pass; the last block to finish turns them into
// exclusive digit offsets and decides which passes run and where each reads
// from / writes to (buffer ids: 0 = input, 1 = alternate, 2 = output; the
// last active pass always writes the output).
__global__ void __launch_bounds__(256) k_sort_hist(const uint32_t* __restrict__ keys, uint32_t N, int begin_bit,
                                                   int end_bit, int passes, SortInfo* info) {
    __shared__ uint32_t sh[kSortMaxPasses][256];
    __shared__ uint32_t s_last;
    const int t = threadIdx.x;
    for (int p = 0; p < passes; ++p) sh[p][t] = 0u;
    __syncthreads();
    // eight keys per thread loaded before any is counted, so their load
    // latencies overlap instead of following each other
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t i = blockIdx.x * blockDim.x + t;
    for (; i < N && N - i > 7u * stride; i += 8u * stride) {
        uint32_t k[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) k[u] = __ldg(keys + i + uint32_t(u) * stride);
#pragma unroll
        for (int u = 0; u < 8; ++u)
            for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][digit_of(k[u], begin_bit, end_bit, p)], 1u);
    }
    for (; i < N; i += stride) {
        const uint32_t k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][digit_of(k, begin_bit, end_bit, p)], 1u);
    }
    __syncthreads();
    for (int p = 0; p < passes; ++p)
        if (sh[p][t]) atomicAdd(&info->hist[p][t], sh[p][t]);
    __threadfence();
    __syncthreads();
    if (t == 0) s_last = (atomicAdd(&info->done, 1u) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    __shared__ uint32_t s_scan[256];
    __shared__ uint32_t s_trivial[kSortMaxPasses];
    for (int p = 0; p < passes; ++p) {
        const uint32_t v = ld_relaxed(&info->hist[p][t]);
        const int trivial = __syncthreads_or(v == N);
        // block-wide exclusive scan of 256 counters
        s_scan[t] = v;
        __syncthreads();
        for (int off = 1; off < 256; off <<= 1) {
            uint32_t add = (t >= off) ? s_scan[t - off] : 0u;
            __syncthreads();
            s_scan[t] += add;
            __syncthreads();
        }
        info->offs[p][t] = s_scan[t] - v;
        if (t == 0) s_trivial[p] = trivial ? 1u : 0u;
        __syncthreads();
    }
    if (t == 0) {
        int active[kSortMaxPasses];
        int T = 0;
        for (int p = 0; p < passes; ++p)
            if (!s_trivial[p]) active[T++] = p;
        for (int p = 0; p < kSortMaxPasses; ++p) info->active[p] = 0u;
        uint32_t prev = 0u;
        for (int a = 0; a < T; ++a) {
            const int p = active[a];
            const uint32_t dst = ((T - 1 - a) % 2 == 0) ? 2u : 1u;
            info->active[p] = 1u;
            info->src[p] = (a == 0) ? 0u : prev;
            info->dst[p] = dst;
            prev = dst;
        }
        info->nactive = uint32_t(T);
    }
}

__device__ __forceinline__ const uint32_t* pick_src_keys(const SortBufs& b, uint32_t id) {
    return id == 0u ? b.keys_in : (id == 1u ? b.keys_alt : b.keys_out);
}
__device__ __forceinline__ const uint32_t* pick_src_vals(const SortBufs& b, uint32_t id) {
    return id == 0u ? b.vals_in : (id == 1u ? b.vals_alt : b.vals_out);
}

template <int kSortItems>
__global__ void __launch_bounds__(kSortThreads) k_sort_pass(SortBufs b, uint32_t N, int begin_bit, int end_bit,
                                                            int pass, int last_pass, SortInfo* info,
                                                            uint32_t* status, uint32_t* err) {
    if (!info->active[pass]) {
        // All passes trivial: the sorted order is the input order.
        if (pass == last_pass && info->nactive == 0u) {
            for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
                b.keys_out[i] = b.keys_in[i];
                b.vals_out[i] = b.vals_in ? b.vals_in[i] : i;
            }
        }
        return;
    }
    __shared__ uint32_t s_hist[kSortWarps][256];
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_tile;
    const int t = threadIdx.x;
    const int lane = t & 31;
    const int warp = t >> 5;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) s_hist[w][t] = 0u;
    if (t == 0) s_tile = atomicAdd(&info->tileCounter[pass], 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t src = info->src[pass];
    const uint32_t dst = info->dst[pass];
    const uint32_t* kin = pick_src_keys(b, src);
    const uint32_t* vin = pick_src_vals(b, src);
    uint32_t* kout = dst == 2u ? b.keys_out : b.keys_alt;
    uint32_t* vout = dst == 2u ? b.vals_out : b.vals_alt;

    const uint32_t base = tile * uint32_t(kSortThreads * kSortItems) + uint32_t(warp) * (32u * kSortItems) + uint32_t(lane);
    uint32_t keys[kSortItems], vals[kSortItems], rank[kSortItems];
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const uint32_t idx = base + uint32_t(j) * 32u;
        const bool valid = idx < N;
        keys[j] = valid ? kin[idx] : 0u;
        vals[j] = valid ? (vin ? vin[idx] : idx) : 0u;
    }
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const uint32_t idx = base + uint32_t(j) * 32u;
        const bool valid = idx < N;
        const uint32_t d = valid ? digit_of(keys[j], begin_bit, end_bit, pass) : 0x100u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const int leader = __ffs(peers) - 1;
        uint32_t prior = 0u;
        if (valid) prior = s_hist[warp][d];
        __syncwarp();
        if (valid && lane == leader) s_hist[warp][d] = prior + __popc(peers);
        __syncwarp();
        rank[j] = prior + __popc(peers & lt);
    }
    __syncthreads();
    // Digit t: exclusive prefix over warps and the tile's total.
    uint32_t run = 0u;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        const uint32_t c = s_hist[w][t];
        s_hist[w][t] = run;
        run += c;
    }
    uint32_t* st = status + size_t(tile) * 256u + t;
    uint32_t excl = 0u;
    if (tile == 0u) {
        st_relaxed(st, kFlagPrefix | run);
    } else {
        st_relaxed(st, kFlagAggregate | run);
        excl = lookback_exclusive(status + t, tile, 256u, err);
        st_relaxed(st, kFlagPrefix | ((excl + run) & kCountMask));
    }
    s_base[t] = info->offs[pass][t] + excl;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const uint32_t idx = base + uint32_t(j) * 32u;
        if (idx < N) {
            const uint32_t d = digit_of(keys[j], begin_bit, end_bit, pass);
            const uint32_t pos = s_base[d] + s_hist[warp][d] + rank[j];
            if (pos < N) {
                kout[pos] = keys[j];
                vout[pos] = vals[j];
            }
        }
    }
}

}  // namespace

size_t sort_temp_bytes(uint32_t N, int num_bits) { return layout_for(N, num_bits).total; }

cudaError_t sort_pairs(void* d_temp, size_t temp_bytes, const uint32_t* keys_in, uint32_t* keys_out,
                       const uint32_t* vals_in, uint32_t* vals_out, uint32_t N, int num_bits, cudaStream_t s,
                       uint32_t* err) {
    if (N == 0) return cudaSuccess;
    if (num_bits < 1) num_bits = 1;
    if (num_bits > 32) num_bits = 32;
    const SortLayout L = layout_for(N, num_bits);
    if (!d_temp || temp_bytes < L.total) return cudaErrorInvalidValue;
    char* base = static_cast<char*>(d_temp);
    SortInfo* info = reinterpret_cast<SortInfo*>(base + L.info_off);
    uint32_t* status = reinterpret_cast<uint32_t*>(base + L.status_off);
    SortBufs b{keys_in, vals_in, reinterpret_cast<uint32_t*>(base + L.keys_alt_off),
               reinterpret_cast<uint32_t*>(base + L.vals_alt_off), keys_out, vals_out};
    if (!err) err = &info->err;
    cudaError_t e = cudaMemsetAsync(base, 0, L.zero_bytes, s);
    if (e != cudaSuccess) return e;
    unsigned hb = blocks_for(N, 256u * 16u);
    if (hb > 608u) hb = 608u;
    if (hb < 1u) hb = 1u;
    k_sort_hist<<<hb, 256, 0, s>>>(keys_in, N, 0, num_bits, L.passes, info);
    for (int p = 0; p < L.passes; ++p) {
        const auto pass = sort_items_for(N) == kSortItemsLarge ? k_sort_pass<kSortItemsLarge> : k_sort_pass<kSortItemsSmall>;
        pass<<<L.tiles, kSortThreads, 0, s>>>(b, N, 0, num_bits, p, L.passes - 1, info,
                                                     status + size_t(p) * L.tiles * 256u, err);
    }
    return cudaGetLastError();
}

}  // namespace pbf
