// pbf_common.cuh - device-side building blocks shared by every PBF kernel.
//
// The arithmetic of each helper restates one reference kernel (cited per
// function) in the same operation order, so results match the reference's
// FP32 kernels to rounding.  Neighbour walks follow the reference order
// (sim/pbf_lambda.cu:49-84): dz, dy, dx over [-reach, reach], cells outside
// [0,dim) skipped, then ascending sorted position.  Because the cells
// dx = -reach..reach of one (dz,dy) row are consecutive keys, their sorted
// ranges are adjacent, so each row is walked as ONE contiguous slot range -
// the same candidates in the same order as the reference's per-cell loop.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "../../include/pbf/parameters.h"
#include "pbf_errors.h"

namespace pbf {

// ---------------------------------------------------------------- errors
// Device-side error word (per sort / per handle).  Kernels never trap: a
// bounded wait that gives up ORs a bit in here and returns.
constexpr uint32_t kErrLookbackTimeout = kErrLookbackTimeoutBit;

// Bounded spin for decoupled look-back: after this many polls the waiting
// block records kErrLookbackTimeout and treats the predecessor as done.
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ------------------------------------------------- TMA bulk copies
// Global -> shared copies on the TMA engine (cp.async.bulk), completing on an
// mbarrier in shared memory.  Both addresses 16-byte aligned, the size a
// multiple of 16 bytes.  Waits on the barrier are bounded.
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(arrivals) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Arrives on the barrier and adds `bytes` to the transfer count its current
// phase waits for.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// Polls phase `parity` of the barrier at most `limit` times; false if it had
// not completed by then.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        __nanosleep(32);
    }
    return false;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ------------------------------------------------ explicitly rounded math
// The reference's kernels are compiled with nvcc's default FMA contraction,
// which fuses some of their multiply-adds.  Which ones depends on the
// surrounding code, so the neighbour arithmetic here spells every operation
// out with round-to-nearest intrinsics (never contracted or reassociated) in
// the reference kernels' fused form: identical results whatever the loop
// structure around them.  The fused form was identified against the
// reference kernels' outputs (every lambda and XSPH velocity of 32,768
// particles bit-identical, lattice and compressed states).
__device__ __forceinline__ float mul_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float div_(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
// a*a + b*b + c*c as the reference's (x*x + y*y + z*z) is fused.
__device__ __forceinline__ float sumsq_(float a, float b, float c) { return fma_(c, c, fma_(a, a, mul_(b, b))); }

// Status word of a decoupled look-back: 2-bit flag | 30-bit count.
constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;

// Walks back over tile statuses [tile-1, tile-2, ...] until an inclusive
// prefix is found; returns the exclusive prefix of `tile`.  Every poll loop is
// bounded by kSpinLimit; *gave_up (when given) is set if one ran out.
__device__ __forceinline__ uint32_t lookback_exclusive(const uint32_t* status, uint32_t tile, uint32_t stride,
                                                       uint32_t* err, uint32_t spin_limit = kSpinLimit,
                                                       bool* gave_up = nullptr) {
    uint32_t excl = 0;
    int64_t k = int64_t(tile) - 1;
    while (k >= 0) {
        const uint32_t* p = status + uint64_t(k) * stride;
        uint32_t v = ld_relaxed(p);
        uint32_t spins = 0;
        while ((v & kFlagMask) == 0u) {
            if (++spins > spin_limit) {
                atomicOr(err, kErrLookbackTimeout);
                if (gave_up) *gave_up = true;
                return excl;
            }
            __nanosleep(32);
            v = ld_relaxed(p);
        }
        excl += v & kCountMask;
        if ((v & kFlagMask) == kFlagPrefix) break;
        --k;
    }
    return excl;
}

// ------------------------------------------------------- predict + clamp
// KIntegratePred (sim/integrate.cu:40-51) followed by the position half of
// KBoundary with e = 0 (sim/boundary.cu:11-25): v' = v + g dt (fused),
// x = p + v' dt (fused), clamp min-then-max per axis, w = 1.  The explicit
// __fmaf_rn pins the rounding so cell keys are reproducible bit for bit.
__device__ __forceinline__ float4 predict_clamped(float4 p, float4 v, float3 g, float dt, const sim::GridBounds& gb) {
    float vx = __fmaf_rn(g.x, dt, v.x);
    float vy = __fmaf_rn(g.y, dt, v.y);
    float vz = __fmaf_rn(g.z, dt, v.z);
    float x = __fmaf_rn(vx, dt, p.x);
    float y = __fmaf_rn(vy, dt, p.y);
    float z = __fmaf_rn(vz, dt, p.z);
    if (x < gb.mins.x) x = gb.mins.x;
    if (y < gb.mins.y) y = gb.mins.y;
    if (z < gb.mins.z) z = gb.mins.z;
    if (x > gb.maxs.x) x = gb.maxs.x;
    if (y > gb.maxs.y) y = gb.maxs.y;
    if (z > gb.maxs.z) z = gb.maxs.z;
    return make_float4(x, y, z, 1.0f);
}

// Full KBoundary on a (position, velocity) pair (sim/boundary.cu:11-25).
__device__ __forceinline__ void boundary_apply(float4& p, float4& v, const sim::GridBounds& gb, float restitution) {
    const float e = fminf(fmaxf(restitution, 0.0f), 1.0f);
    if (p.x < gb.mins.x) { p.x = gb.mins.x; v.x = mul_(v.x, -e); }
    if (p.y < gb.mins.y) { p.y = gb.mins.y; v.y = mul_(v.y, -e); }
    if (p.z < gb.mins.z) { p.z = gb.mins.z; v.z = mul_(v.z, -e); }
    if (p.x > gb.maxs.x) { p.x = gb.maxs.x; v.x = mul_(v.x, -e); }
    if (p.y > gb.maxs.y) { p.y = gb.maxs.y; v.y = mul_(v.y, -e); }
    if (p.z > gb.maxs.z) { p.z = gb.maxs.z; v.z = mul_(v.z, -e); }
    p.w = 1.0f;
    v.w = 0.0f;
}

// KHash (sim/hash_keys.cu:6-27): IEEE divide, floor, clamp to [0,dim-1],
// key = (z*Y + y)*X + x.
__device__ __forceinline__ uint32_t cell_key(float4 p, const sim::GridBounds& gb) {
    int cx = __float2int_rz(floorf(__fdiv_rn(p.x - gb.mins.x, gb.cellSize)));
    int cy = __float2int_rz(floorf(__fdiv_rn(p.y - gb.mins.y, gb.cellSize)));
    int cz = __float2int_rz(floorf(__fdiv_rn(p.z - gb.mins.z, gb.cellSize)));
    cx = max(0, min(cx, gb.dim.x - 1));
    cy = max(0, min(cy, gb.dim.y - 1));
    cz = max(0, min(cz, gb.dim.z - 1));
    return uint32_t((cz * gb.dim.y + cy) * gb.dim.x + cx);
}

__device__ __forceinline__ void decode_key(uint32_t key, int3 dim, int& cx, int& cy, int& cz) {
    cx = int(key % uint32_t(dim.x));
    const uint32_t kdx = key / uint32_t(dim.x);
    cy = int(kdx % uint32_t(dim.y));
    cz = int(kdx / uint32_t(dim.y));
}

// reach = max(1, ceil(h / cs)) (sim/pbf_lambda.cu:47).
__device__ __forceinline__ int neighbour_reach(const sim::DeviceParams& dp) {
    const float cs = dp.grid.cellSize;
    return (cs > 0.f) ? max(1, int(ceilf(dp.kernel.h / cs))) : 1;
}

// Enumerates the (2*reach+1)^2 rows of the stencil in reference order and
// calls visit(k) for every candidate slot k.  rowRange(firstCell, lastCell)
// returns the contiguous slot range [b,e) covering those cells.
template <class RowRange, class Visit>
__device__ __forceinline__ void walk_neighbours(int cx, int cy, int cz, int reach, int3 dim, RowRange&& rowRange,
                                                Visit&& visit) {
    const int x0 = max(cx - reach, 0);
    const int x1 = min(cx + reach, dim.x - 1);
    for (int dz = -reach; dz <= reach; ++dz) {
        const int z = cz + dz;
        if (z < 0 || z >= dim.z) continue;
        for (int dy = -reach; dy <= reach; ++dy) {
            const int y = cy + dy;
            if (y < 0 || y >= dim.y) continue;
            const uint32_t row = uint32_t((z * dim.y + y) * dim.x);
            uint2 r = rowRange(row + uint32_t(x0), row + uint32_t(x1));
            for (uint32_t k = r.x; k < r.y; ++k)
                if (!visit(k)) return;
        }
    }
}

// Two-phase walk of the same candidates in the same order.  All lanes of a
// warp scan in lockstep, one candidate per lane per iteration, testing it
// with hit(k) (cheap) and queueing hits in shared memory (q[j * kStride]).
// Lanes of one cell share their slot ranges, so in lockstep they load the
// same candidates (broadcast) and reach row ends together.  When any lane's
// queue might overflow within the next kChunk candidates, the whole warp
// drains its queues, running body(k) in order; the expensive body thus runs
// only for actual neighbours and with most lanes busy.  At most maxHits
// neighbours are processed (the lambda cap: the reference stops at the first
// `cap` neighbours in walk order).  Every lane of the warp must call this
// (inactive lanes with active = false).
template <int Q, int kStride, bool kCapped = true, class RowRange, class Hit, class Body>
__device__ __forceinline__ void walk_queued(bool active, int cx, int cy, int cz, int reach, int3 dim,
                                            RowRange&& rowRange, uint32_t* q, int maxHits, Hit&& hit,
                                            Body&& body) {
    constexpr int kChunk = 8;
    static_assert(Q > kChunk, "queue must hold more than one chunk");
    const int side = 2 * reach + 1;
    const int nrows = side * side;
    const int x0 = max(cx - reach, 0);
    const int x1 = min(cx + reach, dim.x - 1);
    int ri = -1, total = 0, cnt = 0;
    uint32_t k = 0, e = 0;
    bool done = !active;
    // next in-bounds (dz, dy) row, dz outer, with a non-empty slot range
    auto next_row = [&]() {
        for (;;) {
            if (++ri >= nrows) {
                done = true;
                return;
            }
            const int z = cz + ri / side - reach;
            const int y = cy + ri % side - reach;
            if (z < 0 || z >= dim.z || y < 0 || y >= dim.y) continue;
            const uint32_t row = uint32_t((z * dim.y + y) * dim.x);
            const uint2 r = rowRange(row + uint32_t(x0), row + uint32_t(x1));
            k = r.x;
            e = r.y;
            if (k < e) return;
        }
    };
    if (!done) next_row();
    for (;;) {
        const bool any = __any_sync(0xFFFFFFFFu, !done);
#pragma unroll
        for (int u = 0; u < kChunk; ++u) {
            if (!done) {
                if (hit(k)) {
                    q[cnt * kStride] = k;
                    ++cnt;
                    if (kCapped && ++total >= maxHits) done = true;
                }
                if (!done && ++k >= e) next_row();
            }
        }
        if (!any || __any_sync(0xFFFFFFFFu, cnt > Q - kChunk)) {
            for (int j = 0; j < cnt; ++j) body(q[j * kStride]);
            cnt = 0;
            if (!any) break;
        }
    }
}

// Row ranges from a dense lower-bound table lb[c] = first sorted slot whose
// key >= c (numCells+1 entries).
struct LbRows {
    const uint32_t* __restrict__ lb;
    __device__ __forceinline__ uint2 operator()(uint32_t c0, uint32_t c1) const {
        return make_uint2(__ldg(lb + c0), __ldg(lb + c1 + 1u));
    }
};

// ------------------------------------------------------ neighbour lists
// The walk cell of a particle is its start-of-step cell for the whole step,
// so its candidates (the stencil's slot ranges) are fixed; only positions
// move, and with the displacement clamp on each solver update moves a
// particle by at most maxDisp = disp_clamp_max_h * h.  A list of the
// candidates within R = h + 2 * updates * maxDisp (plus rounding margins) of
// the particle, in walk order, therefore holds every candidate that a pass
// whose positions are within `updates` clamped moves of the list's accepts
// (r^2 <= h^2), and filtering it with the reference's test yields exactly the
// full walk's neighbours in the full walk's order.  (Which passes a list may
// serve, given the box projection after the last update, is decided by the
// host schedule.)  Returns false (lists unusable) when the clamp is off or the
// radius is not finite; builders and users of a list call this with the same
// arguments and so agree.
__device__ __forceinline__ bool list_radius2(const sim::DeviceParams& dp, int updates, float& R2) {
    if (!dp.pbf.enable_disp_clamp || updates < 0) return false;
    const float h = dp.kernel.h;
    const float md = fabsf(dp.pbf.disp_clamp_max_h * h);
    const sim::GridBounds& g = dp.grid;
    // Rounding of x + d: half an ulp of |x| per component; |x| <= box + h +
    // iters * md, and the 0.1% slack on md absorbs the iters * md part for
    // any iteration count below 2000.
    const float box = fmaxf(fmaxf(fmaxf(fabsf(g.mins.x), fabsf(g.maxs.x)), fmaxf(fabsf(g.mins.y), fabsf(g.maxs.y))),
                            fmaxf(fabsf(g.mins.z), fabsf(g.maxs.z)));
    const float perUpdate = md * 1.001f + (box + h) * 4.8e-7f;
    const float R = h * 1.001f + 2.0f * float(updates) * perUpdate;
    R2 = R * R * 1.001f;
    return h > 0.f && isfinite(R2) && R2 >= dp.kernel.h2;
}

// Eight consecutive list entries (32-bit sorted slots or 16-bit indices into
// a staged tile) from a 16-byte aligned address.
__device__ __forceinline__ void load8(const uint32_t* __restrict__ p, uint32_t (&k)[8]) {
    const uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
    const uint4 b = __ldg(reinterpret_cast<const uint4*>(p) + 1);
    k[0] = a.x; k[1] = a.y; k[2] = a.z; k[3] = a.w;
    k[4] = b.x; k[5] = b.y; k[6] = b.z; k[7] = b.w;
}
__device__ __forceinline__ void load8(const uint16_t* __restrict__ p, uint32_t (&k)[8]) {
    const uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
    k[0] = a.x & 0xFFFFu; k[1] = a.x >> 16; k[2] = a.y & 0xFFFFu; k[3] = a.y >> 16;
    k[4] = a.z & 0xFFFFu; k[5] = a.z >> 16; k[6] = a.w & 0xFFFFu; k[7] = a.w >> 16;
}

// A particle's neighbour list: n entries in walk order (E = uint32_t: sorted
// slots; E = uint16_t: indices into the tile staged in shared memory), read
// in chunks of eight: chunk c at lst + c * chunkStride, 16-byte aligned, with
// round_up(n, 8) readable entries.
// `fill` is an index that is safe to read and is used by lanes past their
// list's end (their results are discarded).
template <class E>
struct ListSource {
    const E* __restrict__ lst;
    uint32_t n;
    uint32_t fill;
    // entries from one chunk of eight to the next: 8 for a contiguous list,
    // more for lists interleaved across the slots of a warp
    uint32_t chunkStride = 8;
};

// Eight list entries held as loaded (one or two 16-byte words), unpacked on use.
template <class E>
struct ListChunk;
template <>
struct ListChunk<uint32_t> {
    uint4 a, b;
    __device__ __forceinline__ void load(const uint32_t* __restrict__ p) {
        a = __ldg(reinterpret_cast<const uint4*>(p));
        b = __ldg(reinterpret_cast<const uint4*>(p) + 1);
    }
    __device__ __forceinline__ uint32_t get(int u) const {
        const uint4& w = u < 4 ? a : b;
        const int v = u & 3;
        return v == 0 ? w.x : v == 1 ? w.y : v == 2 ? w.z : w.w;
    }
};
template <>
struct ListChunk<uint16_t> {
    uint4 a;
    __device__ __forceinline__ void load(const uint16_t* __restrict__ p) { a = __ldg(reinterpret_cast<const uint4*>(p)); }
    __device__ __forceinline__ uint32_t get(int u) const {
        const int v = u >> 1;
        const uint32_t w = v == 0 ? a.x : v == 1 ? a.y : v == 2 ? a.z : a.w;
        return (u & 1) ? (w >> 16) : (w & 0xFFFFu);
    }
};

// Lockstep walk over a neighbour list.  Each lane keeps its accepted
// candidates in a ring of Q entries, first in first out, so every particle
// still sums its neighbours in list order.  A lane walks its next chunk of
// eight entries while its ring has room for the chunk (the chunk was loaded
// when the previous one was walked, so its latency hides behind the bodies);
// after each round the warp runs as many bodies as every lane with work left
// has queued (all those lanes busy, two at a time so that their independent
// arithmetic interleaves; each lane still adds its terms in order), and once
// no list is being walked it empties the rings.  kCapped: at most maxHits
// bodies per lane (the reference's neighbour cap), applied once per chunk by
// dropping the hits queued past it; without it no hit count is kept.
template <int Q, int kStride, bool kCapped = true, class E, class QT, class Hit, class Body>
__device__ __forceinline__ void walk_list_queued(bool active, const ListSource<E>& src, QT* q, int maxHits,
                                                 Hit&& hit, Body&& body) {
    constexpr int kChunk = 8;
    constexpr uint32_t kMask = uint32_t(Q - 1);
    static_assert(Q > kChunk && (Q & (Q - 1)) == 0, "the ring holds more than one chunk, a power of two");
    uint32_t head = 0, cnt = 0;
    int total = 0;
    uint32_t e = 0;
    const uint32_t n = src.n;
    bool done = !active || n == 0;
    ListChunk<E> cur;
    if (!done) cur.load(src.lst);
    for (;;) {
        if (!done && cnt <= uint32_t(Q - kChunk)) {
            const uint32_t left = n - e;  // > 0 while the list is being walked
            const uint32_t before = cnt;
#pragma unroll
            for (int u = 0; u < kChunk; ++u) {
                const bool v = uint32_t(u) < left;
                const uint32_t k = v ? cur.get(u) : src.fill;
                const bool h = v && hit(k);
                // cnt + u < Q: the slot is free (live entries are head .. head + cnt - 1)
                q[((head + cnt) & kMask) * kStride] = QT(k);
                cnt += h ? 1u : 0u;
            }
            if (kCapped) {
                // hits past the cap are the last ones queued: drop them
                total += int(cnt - before);
                if (total >= maxHits) {
                    cnt -= uint32_t(total - maxHits);
                    total = maxHits;
                    done = true;
                }
            }
            e += kChunk;
            done = done || e >= n;
            if (!done) cur.load(src.lst + size_t(e >> 3) * src.chunkStride);
        }
        const bool walking = __any_sync(0xFFFFFFFFu, !done);
        // lanes with nothing queued and nothing left to walk do not hold the
        // others back; a lane still walking with an empty ring walks again
        const uint32_t k = walking ? __reduce_min_sync(0xFFFFFFFFu, (done && cnt == 0u) ? 0xFFFFFFFFu : cnt)
                                   : __reduce_max_sync(0xFFFFFFFFu, cnt);
        if (__all_sync(0xFFFFFFFFu, cnt >= k)) {
            uint32_t j = 0;
            for (; j + 2u <= k; j += 2u) {
                const uint32_t ka = q[((head + j) & kMask) * kStride];
                const uint32_t kb = q[((head + j + 1u) & kMask) * kStride];
                body(ka);
                body(kb);
            }
            if (j < k) body(q[((head + j) & kMask) * kStride]);
        } else {
            for (uint32_t j = 0; j < k; ++j)
                if (j < cnt) body(q[((head + j) & kMask) * kStride]);
        }
        const uint32_t m = min(k, cnt);
        head += m;
        cnt -= m;
        if (!walking) break;
    }
}

// Candidate sources of the queued passes: the stencil's rows, or a list.
struct RowSource {
    int cx, cy, cz, reach;
    int3 dim;
    const uint32_t* __restrict__ lb;
};

template <int Q, int kStride, bool kCapped = true, class QT, class Hit, class Body>
__device__ __forceinline__ void walk_source(bool active, const RowSource& r, QT* q, int maxHits, Hit&& hit,
                                            Body&& body) {
    static_assert(std::is_same<QT, uint32_t>::value, "stencil walks queue 32-bit slots");
    walk_queued<Q, kStride, kCapped>(active, r.cx, r.cy, r.cz, r.reach, r.dim, LbRows{r.lb}, q, maxHits, hit, body);
}
template <int Q, int kStride, bool kCapped = true, class E, class QT, class Hit, class Body>
__device__ __forceinline__ void walk_source(bool active, const ListSource<E>& l, QT* q, int maxHits, Hit&& hit,
                                            Body&& body) {
    walk_list_queued<Q, kStride, kCapped>(active, l, q, maxHits, hit, body);
}

// Where the queued passes read a candidate's data: the cell-ordered arrays in
// global memory, or a tile staged in shared memory (x, y, z, lambda) plus
// velocities.
struct GlobalData {
    const float4* __restrict__ pos;
    const float* __restrict__ lam;
    const float4* __restrict__ vel;
    __device__ __forceinline__ float4 p(uint32_t k) const { return __ldg(pos + k); }
    __device__ __forceinline__ float l(uint32_t k, const float4&) const { return __ldg(lam + k); }
    __device__ __forceinline__ float4 v(uint32_t k) const { return __ldg(vel + k); }
};
// The lambda pass's (x, y, z, lambda) per sorted slot: the delta pass reads a
// candidate's position and lambda with one load.
struct PackedData {
    const float4* __restrict__ xl;
    __device__ __forceinline__ float4 p(uint32_t k) const { return __ldg(xl + k); }
    __device__ __forceinline__ float l(uint32_t, const float4& pj) const { return pj.w; }
};
// Staged tile in shared memory: p_[k] = (x, y, z, w) with w = lambda (delta
// passes) or the x velocity (XSPH, whose y and z velocities are in v_[k]).
struct StagedData {
    const float4* p_;
    const float2* v_;
    __device__ __forceinline__ float4 p(uint32_t k) const { return p_[k]; }
    __device__ __forceinline__ float l(uint32_t, const float4& pj) const { return pj.w; }
    __device__ __forceinline__ float4 v(uint32_t k) const {
        const float2 yz = v_[k];
        return make_float4(p_[k].w, yz.x, yz.y, 0.f);
    }
};

// r^2 of a candidate as the reference's neighbour loops compute it
// (sim/pbf_lambda.cu:67-68).
__device__ __forceinline__ float dist2(float4 pi, float4 pj, float& rx, float& ry, float& rz) {
    rx = sub_(pi.x, pj.x);
    ry = sub_(pi.y, pj.y);
    rz = sub_(pi.z, pj.z);
    return sumsq_(rx, ry, rz);
}

// Row ranges from the reference's dense table (start = 0xFFFFFFFF and
// end = 0 for empty cells): min of starts, max of ends.
struct DenseRows {
    const uint32_t* __restrict__ start;
    const uint32_t* __restrict__ end;
    __device__ __forceinline__ uint2 operator()(uint32_t c0, uint32_t c1) const {
        uint32_t b = 0xFFFFFFFFu, e = 0u;
        for (uint32_t c = c0; c <= c1; ++c) {
            uint32_t s = __ldg(start + c), t = __ldg(end + c);
            if (s != 0xFFFFFFFFu && s < t) {
                b = min(b, s);
                e = max(e, t);
            }
        }
        if (b == 0xFFFFFFFFu) b = e = 0u;
        return make_uint2(b, e);
    }
};

// Row ranges from the reference's compact table (sorted unique keys,
// offsets): lower_bound of the first cell (sim/cuda_grid_utils.cuh:34-67),
// then forward over the segments inside the row.
struct CompactRows {
    const uint32_t* __restrict__ uk;
    const uint32_t* __restrict__ off;
    uint32_t M;  // the caller passes min(count, N): a timed-out table's 0xFFFFFFFF stays in bounds
    __device__ __forceinline__ uint2 operator()(uint32_t c0, uint32_t c1) const {
        uint32_t lo = 0, hi = M;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (__ldg(uk + mid) < c0) lo = mid + 1; else hi = mid;
        }
        uint32_t m = lo;
        while (m < M && __ldg(uk + m) <= c1) ++m;
        if (m == lo) return make_uint2(0u, 0u);
        return make_uint2(__ldg(off + lo), __ldg(off + m));
    }
};

// ------------------------------------------------------- arithmetic modes
// The delta pass comes in two modes (a template flag kFast).
//   exact: the reference kernels' operations with explicit rounding, so
//          results are bit-identical to the reference's FP32 kernels, whose
//          s_corr power is CUDA's powf (about 65 instructions, and not
//          correctly rounded: 6.3% of ratio^4 values are an ulp off).
//   fast:  the s_corr power for n = 4 (the default) from error-free products
//          (pow4_compensated, below): ratio^4 to within an ulp, in practice
//          the correctly rounded value, in seven instructions.  Everything
//          else is the exact mode's, so the step stays within the 1e-5
//          relative bars on state; other exponents keep powf.  Two faster
//          variants were measured and dropped: (ratio^2)^2 with a reciprocal
//          of w_q (the last iteration's lambda at 1.05e-5 of the oracle's
//          at 2 iterations), and rsqrtf / reciprocals for the spiky
//          gradient as well (1.8e-5 at 2 iterations, 1.0e-4 at 4).
// x^4 from error-free transformations: q + e = x^2 exactly (e = fma(x, x, -q)),
// r + f = q^2 exactly, and x^4 = q^2 + 2 q e + e^2 = r + (f + 2 q e) with the
// e^2 term below 2^-48 of the result.  The final sum rounds once, so the
// result is within half an ulp of x^4 plus that tiny remainder: correctly
// rounded except within ~2^-24 ulp of a rounding tie.  (x >= 0, as w / w_q is.)
__device__ __forceinline__ float pow4_compensated(float x) {
    const float q = __fmul_rn(x, x);
    const float e = __fmaf_rn(x, x, -q);
    const float r = __fmul_rn(q, q);
    const float f = __fmaf_rn(q, q, -r);
    return __fadd_rn(r, __fmaf_rn(__fmul_rn(2.0f, q), e, f));
}

// Spiky-gradient coefficient -3 spiky (h - r)^2 / max(r, grad_r_eps) of a
// neighbour at r^2 (sim/pbf_lambda.cu:70-74, sim/pbf_delta_apply.cu:70-74).
__device__ __forceinline__ float spiky_coeff(float r2, const sim::DeviceParams& dp) {
    const sim::KernelCoeffs& kc = dp.kernel;
    const float r = sqrt_(r2);
    const float r_safe = fmaxf(r, dp.pbf.grad_r_eps);
    const float t = sub_(kc.h, r);
    return div_(mul_(mul_(-3.0f, kc.spiky), mul_(t, t)), r_safe);
}

// ---------------------------------------------------------------- lambda
// Per-particle constraint multiplier, sim/pbf_lambda.cu:38-107, split into a
// per-neighbour accumulation and a finaliser (the expressions are the
// reference's, evaluated in its order).
struct LambdaAcc {
    float density = 0.f, gx = 0.f, gy = 0.f, gz = 0.f, sumGrad2 = 0.f;
    int contrib = 0;
    uint32_t last = 0;  // candidate index of the last neighbour summed (walks visit them in slot order)
};

__device__ __forceinline__ void lambda_accumulate(LambdaAcc& a, float rx, float ry, float rz, float r2,
                                                  const sim::DeviceParams& dp) {
    const sim::KernelCoeffs& kc = dp.kernel;
    ++a.contrib;
    const float hr2 = sub_(kc.h2, r2);
    a.density = fma_(mul_(mul_(mul_(dp.particleMass, kc.poly6), hr2), hr2), hr2, a.density);
    const float coeff = spiky_coeff(r2, dp);
    const float ax = mul_(coeff, rx), ay = mul_(coeff, ry), az = mul_(coeff, rz);
    a.gx = add_(a.gx, ax);
    a.gy = add_(a.gy, ay);
    a.gz = add_(a.gz, az);
    a.sumGrad2 = add_(a.sumGrad2, sumsq_(ax, ay, az));
}

__device__ __forceinline__ float lambda_finalize(const LambdaAcc& a, const sim::DeviceParams& dp) {
    const sim::PbfTuning& pbf = dp.pbf;
    const float restDensity = dp.restDensity;
    const float gradSum2 = sumsq_(a.gx, a.gy, a.gz);
    const float scale = (restDensity > 0.f) ? div_(dp.particleMass, restDensity) : 0.f;
    const float sum = add_(a.sumGrad2, gradSum2);
    float denom = fma_(mul_(scale, scale), sum, pbf.lambda_denom_eps);
    if (pbf.compliance > 0.f && dp.dt > 0.f) denom = add_(denom, div_(pbf.compliance, mul_(dp.dt, dp.dt)));
    denom = fmaxf(denom, pbf.lambda_denom_eps);
    if (a.contrib < 2 || sum < 1e-12f) return 0.0f;
    const float C = (restDensity > 0.f) ? sub_(div_(a.density, restDensity), 1.f) : 0.f;
    float lam = div_(-C, denom);
    if (!isfinite(lam)) lam = 0.f;
    if (pbf.enable_lambda_clamp) {
        if (fabsf(lam) > pbf.lambda_max_abs) lam = copysignf(pbf.lambda_max_abs, lam);
    }
    return lam;
}

// Single-pass walk (reference layout): fetch(k, j) returns the candidate's
// position and writes its identity j (compared with `self`).  *_acc: the
// neighbour sums before lambda_finalize.
template <class RowRange, class Fetch>
__device__ __forceinline__ LambdaAcc lambda_of_acc(uint32_t self, float4 pi, int cx, int cy, int cz,
                                           const sim::DeviceParams& dp, RowRange&& rows, Fetch&& fetch) {
    LambdaAcc a;
    const int cap = dp.maxNeighbors;
    const bool hasCap = cap > 0;
    walk_neighbours(cx, cy, cz, neighbour_reach(dp), dp.grid.dim, rows, [&](uint32_t k) -> bool {
        if (hasCap && a.contrib >= cap) return false;
        uint32_t j;
        const float4 pj = fetch(k, j);
        if (j == self) return true;
        float rx, ry, rz;
        const float r2 = dist2(pi, pj, rx, ry, rz);
        if (r2 > dp.kernel.h2) return true;
        lambda_accumulate(a, rx, ry, rz, r2, dp);
        a.last = j;
        return true;
    });
    return a;
}

template <class RowRange, class Fetch>
__device__ __forceinline__ float lambda_of(uint32_t self, float4 pi, int cx, int cy, int cz,
                                           const sim::DeviceParams& dp, RowRange&& rows, Fetch&& fetch) {
    return lambda_finalize(lambda_of_acc(self, pi, cx, cy, cz, dp, rows, fetch), dp);
}

// Two-phase walk over cell-ordered positions (slot k is particle k); Src is
// RowSource (the stencil) or a ListSource, Data GlobalData or StagedData.
// Stencil candidates include the particle itself (rejected by slot); lists
// never do.
template <int Q, int kStride, class Src, class Data, class QT>
__device__ __forceinline__ LambdaAcc lambda_queued_acc(bool active, uint32_t s, float4 pi, const Src& src,
                                               const sim::DeviceParams& dp, const Data& data, QT* q) {
    LambdaAcc a;
    const int cap = dp.maxNeighbors;
    const float h2 = dp.kernel.h2;
    constexpr bool kSelf = std::is_same<Src, RowSource>::value;
    walk_source<Q, kStride>(
        active, src, q, cap > 0 ? cap : 0x7FFFFFFF,
        [&](uint32_t k) -> bool {
            float rx, ry, rz;
            return (!kSelf || k != s) && !(dist2(pi, data.p(k), rx, ry, rz) > h2);
        },
        [&](uint32_t k) {
            float rx, ry, rz;
            const float r2 = dist2(pi, data.p(k), rx, ry, rz);
            lambda_accumulate(a, rx, ry, rz, r2, dp);
            a.last = k;
        });
    return a;
}

// s_corr exponent: powf, as the reference (sim/pbf_delta_apply.cu:82).
// With n = 4 exactly (the reference's default) the call names the exponent
// at compile time, which the compiler evaluates with ~19 fewer instructions;
// both forms return the same float for every non-negative input
// (pbf_selftest_powf4 compares them over all 2^31 non-negative bit patterns).
__device__ __forceinline__ float scorr_pow(float ratio, float n) {
    return (n == 4.0f) ? powf(ratio, 4.0f) : powf(ratio, n);
}

// w_q of the tensile-instability term (sim/pbf_delta_apply.cu:40-42).
__device__ __forceinline__ float scorr_wq(const sim::DeviceParams& dp) {
    const float dq = mul_(dp.pbf.scorr_dq_h, dp.kernel.h);
    const float hr2_q = fma_(-dq, dq, dp.kernel.h2);
    return (hr2_q > 0.f) ? mul_(mul_(mul_(dp.kernel.poly6, hr2_q), hr2_q), hr2_q) : dp.pbf.wq_min;
}

// ----------------------------------------------------------------- delta
// Position correction, sim/pbf_delta_apply.cu:40-112.
// One neighbour's term (l_ij, a_ij): the sum is d += l_ij * a_ij per axis.
template <bool kFast = false>
__device__ __forceinline__ float4 delta_term(float rx, float ry, float rz, float r2, float lam_i, float lam_j,
                                             float w_q, const sim::DeviceParams& dp) {
    const sim::KernelCoeffs& kc = dp.kernel;
    const sim::PbfTuning& pbf = dp.pbf;
    const float coeff = spiky_coeff(r2, dp);
    const float ax = mul_(coeff, rx), ay = mul_(coeff, ry), az = mul_(coeff, rz);
    float scorr = 0.0f;
    if (pbf.scorr_enable) {
        const float hr2 = sub_(kc.h2, r2);
        const float w = mul_(mul_(mul_(kc.poly6, hr2), hr2), hr2);
        const float ratio = (w_q > 0.f) ? div_(w, w_q) : 0.0f;
        const float pw = (kFast && pbf.scorr_n == 4.0f) ? pow4_compensated(ratio) : scorr_pow(ratio, pbf.scorr_n);
        scorr = mul_(-pbf.scorr_k, pw);
        if (pbf.scorr_min < 0.f) scorr = fmaxf(scorr, pbf.scorr_min);
    }
    return make_float4(add_(add_(lam_i, lam_j), scorr), ax, ay, az);
}

__device__ __forceinline__ void delta_apply_term(float3& d, float4 term) {
    d.x = fma_(term.x, term.y, d.x);
    d.y = fma_(term.x, term.z, d.y);
    d.z = fma_(term.x, term.w, d.z);
}

template <bool kFast = false>
__device__ __forceinline__ void delta_accumulate(float3& d, float rx, float ry, float rz, float r2, float lam_i,
                                                 float lam_j, float w_q, const sim::DeviceParams& dp) {
    delta_apply_term(d, delta_term<kFast>(rx, ry, rz, r2, lam_i, lam_j, w_q, dp));
}

__device__ __forceinline__ float3 delta_finalize(float3 dsum, const sim::DeviceParams& dp) {
    const sim::PbfTuning& pbf = dp.pbf;
    const float invRest = (dp.restDensity > 0.f) ? div_(1.0f, dp.restDensity) : 0.f;
    float3 d = make_float3(mul_(invRest, dsum.x), mul_(invRest, dsum.y), mul_(invRest, dsum.z));
    if (pbf.enable_relax) {
        d.x = mul_(d.x, pbf.relax_omega);
        d.y = mul_(d.y, pbf.relax_omega);
        d.z = mul_(d.z, pbf.relax_omega);
    }
    if (pbf.enable_disp_clamp) {
        const float maxDisp = mul_(pbf.disp_clamp_max_h, dp.kernel.h);
        const float maxDisp2 = mul_(maxDisp, maxDisp);
        const float len2 = sumsq_(d.x, d.y, d.z);
        if (len2 > maxDisp2) {
            const float len = sqrt_(len2);
            const float s = div_(maxDisp, add_(len, 1e-20f));
            d.x = mul_(d.x, s);
            d.y = mul_(d.y, s);
            d.z = mul_(d.z, s);
        }
    }
    return d;
}

// fetch(k, j, lam_j) returns the candidate position and writes its identity
// and lambda.  *_sum: the neighbour sum before delta_finalize.
template <bool kFast = false, class RowRange, class Fetch>
__device__ __forceinline__ float3 delta_of_sum(uint32_t self, float4 pi, float lam_i, int cx, int cy, int cz,
                                           const sim::DeviceParams& dp, float w_q, RowRange&& rows, Fetch&& fetch) {
    float3 dsum = make_float3(0.f, 0.f, 0.f);
    walk_neighbours(cx, cy, cz, neighbour_reach(dp), dp.grid.dim, rows, [&](uint32_t k) -> bool {
        uint32_t j;
        float lam_j;
        const float4 pj = fetch(k, j, lam_j);
        if (j == self) return true;
        float rx, ry, rz;
        const float r2 = dist2(pi, pj, rx, ry, rz);
        if (r2 > dp.kernel.h2) return true;
        delta_accumulate<kFast>(dsum, rx, ry, rz, r2, lam_i, lam_j, w_q, dp);
        return true;
    });
    return dsum;
}

template <class RowRange, class Fetch>
__device__ __forceinline__ float3 delta_of(uint32_t self, float4 pi, float lam_i, int cx, int cy, int cz,
                                           const sim::DeviceParams& dp, float w_q, RowRange&& rows, Fetch&& fetch) {
    return delta_finalize(delta_of_sum(self, pi, lam_i, cx, cy, cz, dp, w_q, rows, fetch), dp);
}

template <int Q, int kStride, bool kFast = false, class Src, class Data, class QT>
__device__ __forceinline__ float3 delta_queued_sum(bool active, uint32_t s, float4 pi, float lam_i, const Src& src,
                                               const sim::DeviceParams& dp, float w_q, const Data& data, QT* q) {
    float3 dsum = make_float3(0.f, 0.f, 0.f);
    const float h2 = dp.kernel.h2;
    constexpr bool kSelf = std::is_same<Src, RowSource>::value;
    walk_source<Q, kStride, false>(
        active, src, q, 0x7FFFFFFF,
        [&](uint32_t k) -> bool {
            float rx, ry, rz;
            return (!kSelf || k != s) && !(dist2(pi, data.p(k), rx, ry, rz) > h2);
        },
        [&](uint32_t k) {
            float rx, ry, rz;
            const float4 pj = data.p(k);
            const float r2 = dist2(pi, pj, rx, ry, rz);
            delta_accumulate<kFast>(dsum, rx, ry, rz, r2, lam_i, data.l(k, pj), w_q, dp);
        });
    return dsum;
}

// ------------------------------------------------------------------ xsph
// Jacobi XSPH, sim/xsph.cu:39-95.
__device__ __forceinline__ void xsph_accumulate(float3& sum, int& count, float r2, float4 vi, float4 vj,
                                                const sim::DeviceParams& dp) {
    const float hr2 = sub_(dp.kernel.h2, r2);
    const float w = mul_(mul_(mul_(dp.kernel.poly6, hr2), hr2), hr2);
    sum.x = fma_(sub_(vj.x, vi.x), w, sum.x);
    sum.y = fma_(sub_(vj.y, vi.y), w, sum.y);
    sum.z = fma_(sub_(vj.z, vi.z), w, sum.z);
    ++count;
}

__device__ __forceinline__ float4 xsph_finalize(float3 sum, int count, float4 vi, const sim::DeviceParams& dp) {
    float gate = 1.0f;
    if (dp.pbf.xsph_gate_enable) {
        const int nMin = max(0, dp.pbf.xsph_n_min);
        const int nMax = max(nMin + 1, dp.pbf.xsph_n_max);
        const float t = div_(sub_(float(count), float(nMin)), float(nMax - nMin));
        gate = fminf(1.f, fmaxf(0.f, t));
    }
    const float mor = (dp.restDensity > 0.f) ? div_(dp.particleMass, dp.restDensity) : 0.f;
    const float c = mul_(mul_(dp.xsph_c, gate), mor);
    return make_float4(fma_(c, sum.x, vi.x), fma_(c, sum.y, vi.y), fma_(c, sum.z, vi.z), 0.0f);
}

// fetch(k, j, vj) returns the candidate position and writes its identity
// and (old) velocity.
template <class RowRange, class Fetch>
__device__ __forceinline__ float4 xsph_of(uint32_t self, float4 pi, float4 vi, int cx, int cy, int cz,
                                          const sim::DeviceParams& dp, RowRange&& rows, Fetch&& fetch) {
    float3 sum = make_float3(0.f, 0.f, 0.f);
    int count = 0;
    walk_neighbours(cx, cy, cz, neighbour_reach(dp), dp.grid.dim, rows, [&](uint32_t k) -> bool {
        uint32_t j;
        float4 vj;
        const float4 pj = fetch(k, j, vj);
        if (j == self) return true;
        float rx, ry, rz;
        const float r2 = dist2(pi, pj, rx, ry, rz);
        if (r2 > dp.kernel.h2) return true;
        xsph_accumulate(sum, count, r2, vi, vj, dp);
        return true;
    });
    return xsph_finalize(sum, count, vi, dp);
}

template <int Q, int kStride, class Src, class Data, class QT>
__device__ __forceinline__ float4 xsph_queued(bool active, uint32_t s, float4 pi, float4 vi, const Src& src,
                                              const sim::DeviceParams& dp, const Data& data, QT* q) {
    float3 sum = make_float3(0.f, 0.f, 0.f);
    int count = 0;
    const float h2 = dp.kernel.h2;
    constexpr bool kSelf = std::is_same<Src, RowSource>::value;
    walk_source<Q, kStride, false>(
        active, src, q, 0x7FFFFFFF,
        [&](uint32_t k) -> bool {
            float rx, ry, rz;
            return (!kSelf || k != s) && !(dist2(pi, data.p(k), rx, ry, rz) > h2);
        },
        [&](uint32_t k) {
            float rx, ry, rz;
            const float r2 = dist2(pi, data.p(k), rx, ry, rz);
            xsph_accumulate(sum, count, r2, vi, data.v(k), dp);
        });
    return xsph_finalize(sum, count, vi, dp);
}

// XSPH over a list with the body inline (no queue): for light bodies over
// data staged in shared memory, where re-reading candidates is not worth a
// queue.
template <class E, class Data>
__device__ __forceinline__ float4 xsph_list_inline(bool active, float4 pi, float4 vi, const ListSource<E>& src,
                                                   const sim::DeviceParams& dp, const Data& data) {
    float3 sum = make_float3(0.f, 0.f, 0.f);
    int count = 0;
    const float h2 = dp.kernel.h2;
    const uint32_t n = active ? src.n : 0u;
    for (uint32_t e = 0; e < n; e += 8) {
        uint32_t ks[8];
        load8(src.lst + size_t(e >> 3) * src.chunkStride, ks);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (e + uint32_t(u) < n) {
                float rx, ry, rz;
                const uint32_t k = ks[u];
                const float r2 = dist2(pi, data.p(k), rx, ry, rz);
                if (!(r2 > h2)) xsph_accumulate(sum, count, r2, vi, data.v(k), dp);
            }
        }
    }
    return xsph_finalize(sum, count, vi, dp);
}

// Grid size helper.
inline unsigned blocks_for(uint64_t n, unsigned bs) { return unsigned((n + bs - 1) / bs); }

}  // namespace pbf
