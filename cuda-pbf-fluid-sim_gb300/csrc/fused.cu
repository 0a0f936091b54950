// fused.cu - the fused GB300 step.
//
// Phase order is the reference's (sim/phases.cpp:30-117,
// sim/post_ops.cpp:73-85, commit sim/simulator.cpp:144-159); kernels are
// fused where no global barrier separates them:
//   k_predict_keys   predict + boundary(e=0) + cell key          (ids)
//   radix sort       (key, id) -> (key_s, perm)
//   k_gather         re-predicts in cell order (bit-identical to the keyed
//                    prediction), stores step-start positions in cell order
//   cell tables      dense lower-bound table (+ compact table when hashed)
//   k_lambda         per iteration
//   k_delta          per iteration; the last one also applies the post-solve
//                    boundary (e=0) and computes v = (x - p)/dt
//   k_commit         XSPH (Jacobi) + boundary(e) + scatter back to ids
#include "fused.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>

#include "grid.cuh"
#include "pbf_common.cuh"
#include "sort.cuh"

namespace pbf {
namespace {

constexpr int kBS = 256;
// Neighbour walks: a 32-entry ring queue per thread in shared memory,
// column-major so a warp's queue writes hit 32 distinct banks.
constexpr int kQueue = 32;

__global__ void __launch_bounds__(kBS) k_predict_keys(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                      const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                      uint32_t* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const sim::GridBounds g = dpp->grid;
    const float4 x = predict_clamped(pos[i], vel[i], dpp->gravity, dpp->dt, g);
    keys[i] = cell_key(x, g);
}

__global__ void __launch_bounds__(kBS) k_gather(const uint32_t* __restrict__ perm, const float4* __restrict__ pos,
                                                const float4* __restrict__ vel,
                                                const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                float4* __restrict__ pred_s, float4* __restrict__ pos_s) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const uint32_t i = perm[s];
    const float4 p = pos[i];
    pred_s[s] = predict_clamped(p, vel[i], dpp->gravity, dpp->dt, dpp->grid);
    pos_s[s] = p;
}

// ------------------------------------------------------------- scenes
// The list kernels serve one scene (the simulator) or many (the batched
// ensemble) through a scene policy: view(s) gives the parameters of the
// scene sorted slot s belongs to, the first cell of that scene in the global
// cell numbering (keys are global: scene cells are numbered consecutively),
// its solver iteration count and the position updates its neighbour lists
// cover in this pass (< 0: that scene walks the stencil).
struct SceneView {
    const sim::DeviceParams* dp;
    uint32_t cellOffset;
    int iters;
    int listUpdates;
};

struct OneScene {
    const sim::DeviceParams* dp;
    int iters;
    int listUpdates;
    __device__ __forceinline__ uint32_t id(uint32_t) const { return 0u; }
    __device__ __forceinline__ SceneView view(uint32_t) const { return SceneView{dp, 0u, iters, listUpdates}; }
};

struct ManyScenes {
    const SceneInfo* __restrict__ scenes;
    const uint32_t* __restrict__ sceneOfSlot;
    __device__ __forceinline__ uint32_t id(uint32_t s) const { return sceneOfSlot[s]; }
    __device__ __forceinline__ SceneView view(uint32_t s) const {
        const SceneInfo& si = scenes[sceneOfSlot[s]];
        return SceneView{&si.dp, si.cellOffset, si.iters, si.listUpdates};
    }
};

// Neighbour-list buffers of a pass.
struct ListBufs {
    const uint32_t* __restrict__ list;
    const uint32_t* __restrict__ count;
    uint32_t cap;  // 0: no lists
    int staging;   // 0: no tile is staged (all lists hold 32-bit slots)
    // The step's tile plans (kPlanStride uint4 per tile, see plan_tile):
    // the list build writes them, the passes after it load them instead of
    // planning again.  Null: every kernel plans its tiles itself.
    uint4* plans;
};

// Whether slot s's scene has lists this pass (the builder decided the same).
__device__ __forceinline__ bool scene_lists(const SceneView& v, const ListBufs& lb) {
    float R2;
    return lb.cap > 0 && v.listUpdates >= 0 && list_radius2(*v.dp, v.listUpdates, R2);
}

// ------------------------------------------------------------- tiles
// The list passes work on tiles of Sh::kTile consecutive sorted slots, one CTA
// per tile.  When the tile's particles all lie in one scene and one z-plane,
// each of the (2 reach + 1)^2 stencil offsets (dz, dy) is covered by one
// contiguous slot range [start, start + len) (plan_tile_warp): for a tile in
// one row of cells, that row shifted by (dz, dy) over the tile's x range
// widened by reach.  If the ranges hold at most Sh::kStageMax slots, the tile
// is "staged": every list pass copies the ranges into shared memory (range r
// at base[r]) and the lists of its particles hold 16-bit indices into that
// copy, so neighbour reads are shared-memory gathers.
// Other tiles' lists hold 32-bit sorted slots read from global memory.  The
// plan depends only on the sorted keys, the lower-bound table and the
// scenes, so the list builder and every list pass derive the same one.
constexpr int kPlanRows = 32;

// A tile shape the list passes (and the list build, which must plan the same
// tiles) are compiled for: slots per tile (= threads per CTA), stage slots,
// and the CTAs per SM that the shape's shared memory allows, which the launch
// bounds pass on so that the register budget matches that occupancy.  The
// shapes give identical results (only which tiles are staged differs); the
// autotuner picks one by timing.
//
// Shared memory of the list passes.  lambda / delta: the stage (kStageMax
// float4) then a queue of 16-bit stage indices (kQueue x kTile) for staged
// tiles; tiles that are not staged keep 32-bit queues in the stage area.
// XSPH: the stage as float4 (x, y, z, vx) plus float2 (vy, vz), its queue in
// the stage area likewise.  In a staged tile a warp whose lists overflowed
// walks the stencil in one pass, without a queue.
template <int T, int S, int MinSolve, int MinCommit>
struct TileShape {
    static constexpr int kTile = T;
    static constexpr int kStageMax = S;
    static constexpr int kMinSolve = MinSolve;
    static constexpr int kMinCommit = MinCommit;
    static constexpr size_t kStageBytes = size_t(S) * sizeof(float4);
    static constexpr size_t kSolveSmem = kStageBytes + size_t(kQueue) * T * sizeof(uint16_t);
    static constexpr size_t kCommitSmem = kStageBytes + size_t(S) * sizeof(float2);
    static_assert(T % 32 == 0 && T <= 1024, "tiles are whole warps of one CTA");
    static_assert(S <= 32768, "staged indices are 16-bit");
    static_assert(size_t(kQueue) * T * sizeof(uint32_t) <= kStageBytes, "32-bit queues fit in the stage area");
};
using TileShape0 = TileShape<128, 1536, 6, 6>;
using TileShape1 = TileShape<64, 1024, 10, 8>;
using TileShape2 = TileShape<128, 2048, 5, 4>;
using TileShape3 = TileShape<256, 3072, 3, 3>;

struct TilePlan {
    uint64_t bar;  // completes when the staged rows have landed in shared memory
    uint32_t start[kPlanRows];
    uint32_t base[kPlanRows];
    uint32_t len[kPlanRows];
    uint32_t total;
    int nrows;
    int staged;
    int lists;  // the tile's scene has lists this pass
};

// A tile's plan as one warp holds it: lane r holds row r's range and stage
// base.  Called by a whole warp.
struct WarpPlan {
    uint32_t start, base, len;  // this lane's row
    uint32_t total;
    int nrows;
    bool staged;
    bool lists;
};

template <class Sh, class Scenes>
__device__ WarpPlan plan_tile_warp(const uint32_t* __restrict__ key_s, const uint32_t* __restrict__ lb,
                                   const Scenes& S, const ListBufs& lbuf, uint32_t t0, uint32_t N) {
    const int lane = int(threadIdx.x & 31u);
    const uint32_t tl = min(t0 + uint32_t(Sh::kTile), N) - 1u;
    const SceneView v = S.view(t0);
    const sim::DeviceParams& dp = *v.dp;
    const int3 dim = dp.grid.dim;
    const bool oneScene = S.id(t0) == S.id(tl);
    int xf, yf, zf, xl = 0, yl = -1, zl = -1;
    decode_key(key_s[t0] - v.cellOffset, dim, xf, yf, zf);
    if (oneScene) decode_key(key_s[tl] - v.cellOffset, dim, xl, yl, zl);
    const int reach = neighbour_reach(dp);
    const int side = 2 * reach + 1;
    WarpPlan w;
    w.nrows = side * side;
    w.lists = scene_lists(v, lbuf);
    // Tiles within one z-plane: lane r stages stencil offset r = (dz, dy) as
    // the cells from (y0 + dy, x0 - reach) to (y1 + dy, x1 + reach) of plane
    // z + dz, consecutive in sorted order, where (x0, y0) and (x1, y1) are the
    // first and last particles' cells.  Every particle of the tile finds its
    // row (dz, dy) inside: for a one-row tile (y0 = y1) the range is that row
    // over the tile's x-extent, for a tile across rows it runs from the first
    // row's tail over any whole rows to the last row's head.
    const bool samePlane = oneScene && zf == zl && w.nrows <= kPlanRows;
    w.start = 0;
    w.len = 0;
    if (samePlane && lane < w.nrows) {
        const int z = zf + lane / side - reach;
        const int dy = lane % side - reach;
        const int ya = yf + dy, yb = yl + dy;
        if (z >= 0 && z < dim.z && yb >= 0 && ya < dim.y) {
            const uint32_t* slb = lb + v.cellOffset;
            const uint32_t plane = uint32_t(z * dim.y);
            const uint32_t first = ya >= 0 ? (plane + uint32_t(ya)) * uint32_t(dim.x) + uint32_t(max(xf - reach, 0))
                                           : plane * uint32_t(dim.x);
            const uint32_t last = yb < dim.y
                                      ? (plane + uint32_t(yb)) * uint32_t(dim.x) + uint32_t(min(xl + reach, dim.x - 1))
                                      : (plane + uint32_t(dim.y)) * uint32_t(dim.x) - 1u;
            w.start = __ldg(slb + first);
            w.len = __ldg(slb + last + 1u) - w.start;
        }
    }
    uint32_t incl = w.len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += t;
    }
    w.total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    w.base = incl - w.len;
    w.staged = samePlane && w.total <= uint32_t(Sh::kStageMax);
    return w;
}

// A tile's plan in global memory: uint4 0 = (total, nrows, staged, 0),
// uint4 1 + r = (start, base, len, 0) of row r.  The plan depends only on the
// step's sorted keys, lower-bound table and tile shape, so every pass of a
// step would compute the same one.
constexpr int kPlanStride = kPlanRows + 1;

// How plan_and_issue gets the CTA's plan.
enum PlanMode { kPlanCompute = 0, kPlanStore = 1, kPlanLoad = 2 };

// The plan in shared memory for a CTA (written by warp 0): computed, and with
// kPlanStore also written to the step's plan array; or, with kPlanLoad,
// loaded from there (row ranges, total, staged; the lists flag is this
// pass's own).
template <class Sh, class Scenes>
__device__ void plan_tile(TilePlan& P, const uint32_t* __restrict__ key_s, const uint32_t* __restrict__ lb,
                          const Scenes& S, const ListBufs& lbuf, uint32_t t0, uint32_t N, PlanMode mode) {
    const int lane = int(threadIdx.x & 31u);
    uint4* tp = lbuf.plans ? lbuf.plans + size_t(t0 / uint32_t(Sh::kTile)) * kPlanStride : nullptr;
    if (mode == kPlanLoad && tp) {
        const uint4 row = __ldg(tp + 1 + lane);
        const uint4 head = __ldg(tp);
        P.start[lane] = row.x;
        P.base[lane] = row.y;
        P.len[lane] = row.z;
        if (lane == 0) {
            P.total = head.x;
            P.nrows = int(head.y);
            P.staged = int(head.z);
            P.lists = scene_lists(S.view(t0), lbuf) ? 1 : 0;
        }
        return;
    }
    const WarpPlan w = plan_tile_warp<Sh>(key_s, lb, S, lbuf, t0, N);
    P.start[lane] = w.start;
    P.base[lane] = w.base;
    P.len[lane] = w.len;
    if (lane == 0) {
        P.total = w.total;
        P.nrows = w.nrows;
        P.staged = w.staged ? 1 : 0;
        P.lists = w.lists ? 1 : 0;
    }
    if (mode == kPlanStore && tp) {
        tp[1 + lane] = make_uint4(w.start, w.base, w.len, 0u);
        if (lane == 0) tp[0] = make_uint4(w.total, uint32_t(w.nrows), w.staged ? 1u : 0u, 0u);
    }
}

// The list length of slot sc, loaded before the tile's plan so that its
// latency overlaps the plan's (0 without lists).
__device__ __forceinline__ uint32_t list_count(const ListBufs& lbuf, uint32_t sc) {
    return lbuf.cap ? __ldg(lbuf.count + sc) : 0u;
}

// Whether this warp walks its lists: every lane that walks has lists in its
// scene and none of them overflowed (count: list_count of the lane's slot).
// Every lane must call it.
__device__ __forceinline__ bool warp_lists_fit(const ListBufs& lbuf, bool active, bool laneLists, uint32_t count,
                                               uint32_t& n) {
    n = 0;
    if (!__all_sync(0xFFFFFFFFu, !active || laneLists)) return false;
    n = active ? count : 0u;
    return !__any_sync(0xFFFFFFFFu, n > lbuf.cap);
}

__device__ __forceinline__ RowSource row_source(const uint32_t* __restrict__ key_s, const uint32_t* __restrict__ lb,
                                                const SceneView& v, uint32_t sc) {
    RowSource r;
    decode_key(key_s[sc] - v.cellOffset, v.dp->grid.dim, r.cx, r.cy, r.cz);
    r.reach = neighbour_reach(*v.dp);
    r.dim = v.dp->grid.dim;
    r.lb = lb + v.cellOffset;
    return r;
}

// Plans the CTA's tile and, when it is staged and its scene has lists, starts
// copying the staged rows into shared memory (sp[base[r] + i] = src[start[r]
// + i]; src: positions, or the lambda pass's (x, y, z, lambda) for the delta
// pass): thread 0 issues one TMA bulk copy per row, completing on the plan's
// barrier, while the other threads go on with their own loads.  Returns
// whether the tile is staged.  CTA-uniform; every thread calls it, and every
// thread then calls stage_finish before reading the stage.
template <class Sh, class Scenes>
__device__ __forceinline__ bool plan_and_issue(TilePlan& P, const uint32_t* __restrict__ key_s,
                                               const uint32_t* __restrict__ lb, const Scenes& S,
                                               const ListBufs& lbuf, uint32_t t0, uint32_t N,
                                               const float4* __restrict__ src, float4* sp,
                                               PlanMode mode = kPlanLoad) {
    // no lists, or lists of 32-bit slots only (the adjoint's replay): no tile
    // is staged, and no plan is needed
    if (lbuf.cap == 0 || !lbuf.staging) return false;
    if (threadIdx.x < 32) plan_tile<Sh>(P, key_s, lb, S, lbuf, t0, N, mode);
    if (threadIdx.x == 0) mbar_init(&P.bar, 1);
    __syncthreads();
    const bool staged = P.staged && P.lists && lbuf.staging;
    if (staged && threadIdx.x == 0) {
        // rows are float4 ranges: 16-byte aligned, sizes multiples of 16
        mbar_arrive_expect_tx(&P.bar, P.total * uint32_t(sizeof(float4)));
        for (int r = 0; r < P.nrows; ++r)
            if (P.len[r]) bulk_copy_g2s(sp + P.base[r], src + P.start[r], P.len[r] * uint32_t(sizeof(float4)), &P.bar);
    }
    return staged;
}

// Waits (bounded) for the staged rows, then, with vel given, fills in the
// rest of the stage: w = vel[k].x and sv[i] = (vel[k].y, vel[k].z).  A wait
// that gives up sets kErrStageTimeoutBit and waits once more (also bounded)
// so that no copy is still landing when the tile moves on; if that wait gives
// up too, in any thread, the stage is not used: the function returns false
// and the tile's warps walk the stencil from global memory instead.
// CTA-uniform; every thread calls it.
template <class Sh>
__device__ __forceinline__ bool stage_finish(TilePlan& P, bool staged, const float4* __restrict__ vel, float4* sp,
                                             float2* sv, uint32_t* err) {
    if (!staged) return true;
    bool landed = mbar_wait_bounded(&P.bar, 0u, kSpinLimit);
    if (!landed) {
        if (err) atomicOr(err, kErrStageTimeoutBit);
        landed = mbar_wait_bounded(&P.bar, 0u, kSpinLimit);
    }
    if (__syncthreads_or(!landed)) return false;
    if (!vel) return true;
    for (int r = 0; r < P.nrows; ++r) {
        const uint32_t st = P.start[r], bs = P.base[r], len = P.len[r];
        for (uint32_t i = threadIdx.x; i < len; i += Sh::kTile) {
            const float4 v = __ldg(vel + st + i);
            reinterpret_cast<float*>(sp + bs + i)[3] = v.x;
            sv[bs + i] = make_float2(v.y, v.z);
        }
    }
    __syncthreads();
    return true;
}

// Packed two-lane FP32 arithmetic (Blackwell f32x2): the list test of two
// particles against one candidate in half the instructions.  Each half is an
// ordinary round-to-nearest FP32 operation.
__device__ __forceinline__ unsigned long long pk2(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 upk2(unsigned long long v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Layout of the lists.  Slot s owns cap 32-bit words of the list buffer.
// Lists of tiles that are not staged hold sorted slots there, contiguously
// (list + s * cap).  Lists of staged tiles hold 16-bit stage indices (2 cap of
// room) and are interleaved by groups of 32 slots: the 32 lists of a group
// share the group's 64 cap 16-bit entries, chunk c (entries 8c .. 8c + 7) of
// slot s sitting at c * 256 + (s % 32) * 8.  A warp walking the same chunk of
// its 32 lists then loads 512 contiguous bytes instead of 32 scattered 16-byte
// pieces.  Tiles are whole groups, so a group holds one format; the buffer
// holds a whole number of groups (allocations round the slots up to 32).
constexpr uint32_t kListGroup = 32;
constexpr uint32_t kList16ChunkStride = 8 * kListGroup;  // entries between a list's chunks
__device__ __forceinline__ uint16_t* list16_base(uint32_t* list, uint32_t cap, uint32_t s) {
    return reinterpret_cast<uint16_t*>(list) + size_t(s / kListGroup) * (2u * kListGroup * cap) +
           (s % kListGroup) * 8u;
}
__device__ __forceinline__ const uint16_t* list16_base(const uint32_t* list, uint32_t cap, uint32_t s) {
    return list16_base(const_cast<uint32_t*>(list), cap, s);
}
// Position of entry j of an interleaved 16-bit list.
__device__ __forceinline__ uint32_t list16_at(uint32_t j) { return (j >> 3) * kList16ChunkStride + (j & 7u); }

// One particle's list being written by a warp: hits of a 32-candidate step
// are compacted with a ballot into consecutive entries.
struct ListWriter {
    uint32_t* out;    // the particle's 32-bit list (tiles that are not staged)
    uint16_t* out16;  // its interleaved 16-bit list (staged tiles)
    uint32_t cnt;
    __device__ __forceinline__ void emit(bool in, uint32_t k, uint32_t shift, uint32_t cap, bool staged,
                                         uint32_t lt) {
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, in);
        const uint32_t at = cnt + __popc(m & lt);
        if (in && at < cap) {
            if (staged)
                out16[list16_at(at)] = uint16_t(k + shift);
            else
                out[at] = k;
        }
        cnt += __popc(m);
    }
    // Staged tile with cap >= 32: a list of 16-bit entries has 2 cap of room,
    // so while cnt <= cap (a warp-uniform test) an emit writes below cap + 32
    // and needs no bound per lane; entries past cap are never read (the count
    // then exceeds cap and the warp walks the stencil).
    __device__ __forceinline__ void emit16(bool in, uint32_t k, uint32_t shift, uint32_t cap, uint32_t lt) {
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, in);
        if (in && cnt <= cap) out16[list16_at(cnt + __popc(m & lt))] = uint16_t(k + shift);
        cnt += __popc(m);
    }
};

__device__ __forceinline__ ListWriter list_writer(uint32_t* list, uint32_t cap, uint32_t s) {
    return ListWriter{list + size_t(s) * cap, list16_base(list, cap, s), 0u};
}

// One row of the list build for G particles of one cell: candidates [b, e),
// 32 per step.  kSlack: staged tile with cap >= 32 (ListWriter::emit16).
template <int G, bool kSlack>
__device__ __forceinline__ void build_row(const float4* __restrict__ pred, const uint32_t (&sl)[G],
                                          const float4& p0, const unsigned long long (&px)[G / 2],
                                          const unsigned long long (&py)[G / 2],
                                          const unsigned long long (&pz)[G / 2], int used, uint32_t b, uint32_t e,
                                          uint32_t shift, float R2, uint32_t cap, bool staged, uint32_t lt,
                                          uint32_t lane, ListWriter (&w)[G]) {
#pragma unroll 2
    for (uint32_t c = b; c < e; c += 32u) {
        const uint32_t k = c + lane;
        const bool valid = k < e;
        const float4 pj = valid ? __ldg(pred + k) : p0;
        const unsigned long long jx = pk2(pj.x, pj.x), jy = pk2(pj.y, pj.y), jz = pk2(pj.z, pj.z);
#pragma unroll
        for (int h = 0; h < G / 2; ++h) {
            // r^2 = rz^2 + (rx^2 + ry^2), as the neighbour passes compute it
            const unsigned long long dx = sub2(px[h], jx), dy = sub2(py[h], jy), dz = sub2(pz[h], jz);
            const float2 r2 = upk2(fma2(dz, dz, fma2(dx, dx, mul2(dy, dy))));
            const bool in0 = valid && k != sl[2 * h] && !(r2.x > R2);
            const bool in1 = valid && k != sl[2 * h + 1] && !(r2.y > R2);
            if (kSlack)
                w[2 * h].emit16(in0, k, shift, cap, lt);
            else
                w[2 * h].emit(in0, k, shift, cap, staged, lt);
            if (2 * h + 1 < used) {
                if (kSlack)
                    w[2 * h + 1].emit16(in1, k, shift, cap, lt);
                else
                    w[2 * h + 1].emit(in1, k, shift, cap, staged, lt);
            }
        }
    }
}

// The row walk of the list build for G particles of one cell (G even;
// particle g emits only when g < used): each candidate is loaded once and
// tested against the particles two at a time with packed arithmetic.
template <int G, bool kSlack>
__device__ __forceinline__ void build_rows(const float4* __restrict__ pred, const uint32_t (&sl)[G],
                                           const float4 (&pp)[G], int used, int nrows, uint32_t rb, uint32_t re,
                                           uint32_t planShift, float R2, uint32_t cap, bool staged, uint32_t lt,
                                           uint32_t lane, ListWriter (&w)[G]) {
    static_assert(G % 2 == 0, "particles are tested in pairs");
    unsigned long long px[G / 2], py[G / 2], pz[G / 2];
#pragma unroll
    for (int h = 0; h < G / 2; ++h) {
        px[h] = pk2(pp[2 * h].x, pp[2 * h + 1].x);
        py[h] = pk2(pp[2 * h].y, pp[2 * h + 1].y);
        pz[h] = pk2(pp[2 * h].z, pp[2 * h + 1].z);
    }
    for (int rr = 0; rr < nrows; ++rr) {
        const uint32_t b = __shfl_sync(0xFFFFFFFFu, rb, rr);
        const uint32_t e = __shfl_sync(0xFFFFFFFFu, re, rr);
        // staged tiles have nrows <= 32, so the plan's lane rr is row rr
        const uint32_t shift = __shfl_sync(0xFFFFFFFFu, planShift, rr);
        build_row<G, kSlack>(pred, sl, pp[0], px, py, pz, used, b, e, shift, R2, cap, staged, lt, lane, w);
    }
}

// Builds the neighbour lists: a warp takes its 32 particles one at a time
// (four or two at a time when consecutive particles share a cell, testing
// them against each candidate with packed arithmetic), 32 candidates per step,
// and a ballot compacts the candidates within the list radius into the
// particle's list in walk order (coalesced stores).  Entries are 16-bit
// stage indices in staged tiles, 32-bit sorted slots otherwise; each warp
// derives its tile's plan itself.  The stencil's row ranges are reused while
// consecutive particles share a cell.  A particle whose scene has no lists
// gets the count cap + 1 (its warp walks the stencil).
template <class Scenes, class Sh>
__device__ __forceinline__ void build_lists_warp(uint32_t s0, const float4* __restrict__ pred,
                                                 const uint32_t* __restrict__ key_s, const uint32_t* __restrict__ lb,
                                                 const Scenes& S, uint32_t N, const ListBufs& lbuf,
                                                 uint32_t* __restrict__ list, uint32_t* __restrict__ count,
                                                 uint32_t* __restrict__ stats) {
    const uint32_t lane = threadIdx.x & 31u;
    if (s0 >= N) return;  // warp-uniform
    const uint32_t cap = lbuf.cap;
    const WarpPlan plan = plan_tile_warp<Sh>(key_s, lb, S, lbuf, s0 - s0 % uint32_t(Sh::kTile), N);
    const bool staged = plan.staged && lbuf.staging;
    const bool slack = staged && cap >= 32u;  // ListWriter::emit16
    const uint32_t planShift = plan.base - plan.start;  // lane r: stage index of slot k in row r is k + shift
    const uint32_t lt = lanemask_lt();
    uint32_t longest = 0, overflowed = 0;
    const uint32_t pend = min(N - s0, 32u);
    // rows of the cell last set up: lane r < nrows holds row r's range
    uint32_t cachedKey = 0xFFFFFFFFu, rb = 0, re = 0;
    int nrows = 0;
    bool flat = false;
    uint32_t T = 0, startOf = 0, endOf = 0;  // flattened rows: lane r < 9 holds row r's start and end
    float R2 = 0.f;
    for (uint32_t p = 0; p < pend;) {
        const uint32_t s = s0 + p;
        const uint32_t key = key_s[s];
        const SceneView v = S.view(s);  // warp-uniform: one cell at a time
        const sim::DeviceParams& dp = *v.dp;
        if (key != cachedKey) {
            if (v.listUpdates < 0 || !list_radius2(dp, v.listUpdates, R2)) {
                if (lane == 0) count[s] = cap + 1u;
                ++p;
                continue;
            }
            const int reach = neighbour_reach(dp);
            const int side = 2 * reach + 1;
            nrows = side * side;
            const int3 dim = dp.grid.dim;
            int cx, cy, cz;
            decode_key(key - v.cellOffset, dim, cx, cy, cz);
            const int x0 = max(cx - reach, 0);
            const int x1 = min(cx + reach, dim.x - 1);
            // rows beyond 32 (reach > 2) are set up per batch below
            rb = re = 0;
            const int r = int(lane);
            if (r < nrows) {
                const int z = cz + r / side - reach;
                const int y = cy + r % side - reach;
                if (z >= 0 && z < dim.z && y >= 0 && y < dim.y) {
                    const uint32_t row = uint32_t((z * dim.y + y) * dim.x);
                    rb = __ldg(lb + v.cellOffset + row + uint32_t(x0));
                    re = __ldg(lb + v.cellOffset + row + uint32_t(x1) + 1u);
                }
            }
            flat = false;
            if (nrows == 9) {
                // Short rows (sparse regions): walk the 9 rows as one
                // flattened sequence, 32 candidates per step whatever the row
                // lengths, when that takes fewer steps' worth of instructions
                // than row by row.
                const uint32_t len = re - rb;
                uint32_t end = len;  // inclusive prefix: end of row r in the flattened sequence
#pragma unroll
                for (int o = 1; o < 16; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, end, o);
                    if (int(lane) >= o) end += t;
                }
                T = __shfl_sync(0xFFFFFFFFu, end, 8);
                const uint32_t rowSteps = __reduce_add_sync(0xFFFFFFFFu, (len + 31u) >> 5);
                flat = ((T + 31u) >> 5) * 2u < rowSteps;
                if (flat) {
                    endOf = end;
                    startOf = end - len;
                }
            }
            cachedKey = key;
        }
        // up to three more particles of the same cell go along (the row walk only)
        const bool quad = !flat && nrows <= 32 && p + 3 < pend && key_s[s + 3] == key;
        const bool pair = !flat && nrows <= 32 && !quad && p + 1 < pend && key_s[s + 1] == key;
        const int used = quad ? 4 : pair ? 2 : 1;
        if (quad) {
            uint32_t sl[4];
            float4 pp[4];
            ListWriter w[4];
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                sl[g] = s + uint32_t(g);
                pp[g] = pred[sl[g]];
                w[g] = list_writer(list, cap, sl[g]);
            }
            if (slack)
                build_rows<4, true>(pred, sl, pp, 4, nrows, rb, re, planShift, R2, cap, staged, lt, lane, w);
            else
                build_rows<4, false>(pred, sl, pp, 4, nrows, rb, re, planShift, R2, cap, staged, lt, lane, w);
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                if (lane == 0) count[sl[g]] = w[g].cnt;
                longest = max(longest, w[g].cnt);
                overflowed += w[g].cnt > cap ? 1u : 0u;
            }
            p += 4u;
            continue;
        }
        const uint32_t sB = pair ? s + 1 : s;
        const float4 pa = pred[s], pb = pred[sB];
        ListWriter wa = list_writer(list, cap, s);
        ListWriter wb = list_writer(list, cap, sB);
        if (flat) {
            for (uint32_t c = 0; c < T; c += 32u) {
                const uint32_t vi = c + lane;
                uint32_t row = 0;
#pragma unroll
                for (int q = 0; q < 8; ++q) row += (__shfl_sync(0xFFFFFFFFu, endOf, q) <= vi) ? 1u : 0u;
                const uint32_t k = __shfl_sync(0xFFFFFFFFu, rb, int(row)) +
                                   (vi - __shfl_sync(0xFFFFFFFFu, startOf, int(row)));
                const uint32_t shift = __shfl_sync(0xFFFFFFFFu, planShift, int(row));
                bool in = false;
                if (vi < T) {
                    float rx, ry, rz;
                    in = k != s && !(dist2(pa, __ldg(pred + k), rx, ry, rz) > R2);
                }
                wa.emit(in, k, shift, cap, staged, lt);
            }
        } else if (nrows <= 32) {
            const uint32_t sl[2] = {s, sB};
            const float4 pp[2] = {pa, pb};
            ListWriter w[2] = {wa, wb};
            if (slack)
                build_rows<2, true>(pred, sl, pp, used, nrows, rb, re, planShift, R2, cap, staged, lt, lane, w);
            else
                build_rows<2, false>(pred, sl, pp, used, nrows, rb, re, planShift, R2, cap, staged, lt, lane, w);
            wa = w[0];
            wb = w[1];
        } else {
            // reach > 2: rows in batches of 32, one particle at a time
            const int reach = neighbour_reach(dp);
            const int side = 2 * reach + 1;
            const int3 dim = dp.grid.dim;
            int cx, cy, cz;
            decode_key(key - v.cellOffset, dim, cx, cy, cz);
            const int x0 = max(cx - reach, 0);
            const int x1 = min(cx + reach, dim.x - 1);
            for (int r0 = 0; r0 < nrows; r0 += 32) {
                const int r = r0 + int(lane);
                uint32_t bb = 0, ee = 0;
                if (r < nrows) {
                    const int z = cz + r / side - reach;
                    const int y = cy + r % side - reach;
                    if (z >= 0 && z < dim.z && y >= 0 && y < dim.y) {
                        const uint32_t row = uint32_t((z * dim.y + y) * dim.x);
                        bb = __ldg(lb + v.cellOffset + row + uint32_t(x0));
                        ee = __ldg(lb + v.cellOffset + row + uint32_t(x1) + 1u);
                    }
                }
                const int nr = min(32, nrows - r0);
                for (int rr = 0; rr < nr; ++rr) {
                    const uint32_t b = __shfl_sync(0xFFFFFFFFu, bb, rr);
                    const uint32_t e = __shfl_sync(0xFFFFFFFFu, ee, rr);
                    for (uint32_t c = b; c < e; c += 32u) {
                        const uint32_t k = c + lane;
                        bool in = false;
                        if (k < e) {
                            float rx, ry, rz;
                            in = k != s && !(dist2(pa, __ldg(pred + k), rx, ry, rz) > R2);
                        }
                        wa.emit(in, k, 0u, cap, false, lt);  // nrows > 32: never staged
                    }
                }
            }
        }
        if (lane == 0) {
            count[s] = wa.cnt;
            if (pair) count[sB] = wb.cnt;
        }
        longest = max(longest, pair ? max(wa.cnt, wb.cnt) : wa.cnt);
        overflowed += (wa.cnt > cap ? 1u : 0u) + (pair && wb.cnt > cap ? 1u : 0u);
        p += pair ? 2u : 1u;
    }
    if (lane == 0 && stats) {
        atomicMax(stats, longest);
        if (overflowed) atomicAdd(stats + 1, overflowed);
    }
}

// The list build of a whole tile (one CTA of Sh::kTile threads).  A staged
// tile copies its stencil rows into shared memory, as the passes do, and
// every thread builds its own particle's list from there: for each of its
// rows it tests the row's cells (the slot range from the lower-bound table,
// inside the tile's staged range) against its position, in walk order, and
// emits the stage indices of the candidates within the list radius, eight
// 16-bit entries to a 16-byte store.  That is a few instructions per
// candidate instead of a warp step per 32 candidates of one particle.  The r^2
// test is the passes' (dist2), so the lists are the same.  Tiles that are not
// staged, or whose staging wait gave up, are built warp by warp from global
// memory (build_lists_warp), which writes the same entries.
template <class Scenes, class Sh>
__global__ void __launch_bounds__(Sh::kTile) k_build_lists_tiled(const float4* __restrict__ pred,
                                                                 const uint32_t* __restrict__ key_s,
                                                                 const uint32_t* __restrict__ lb, Scenes S,
                                                                 uint32_t N, ListBufs lbuf,
                                                                 uint32_t* __restrict__ list,
                                                                 uint32_t* __restrict__ count,
                                                                 uint32_t* __restrict__ stats,
                                                                 uint32_t* __restrict__ err) {
    extern __shared__ float4 smem[];
    __shared__ TilePlan P;
    __shared__ uint32_t s_longest, s_over;
    float4* sp = smem;
    const uint32_t t0 = blockIdx.x * Sh::kTile;
    // the passes of this step load the plan this build stores
    const bool staged = plan_and_issue<Sh>(P, key_s, lb, S, lbuf, t0, N, pred, sp, kPlanStore);
    const bool stageOk = stage_finish<Sh>(P, staged, nullptr, sp, nullptr, err);
    if (!staged || !stageOk) {  // CTA-uniform
        build_lists_warp<Scenes, Sh>(t0 + (threadIdx.x & ~31u), pred, key_s, lb, S, N, lbuf, list, count, stats);
        return;
    }
    if (threadIdx.x == 0) {
        s_longest = 0;
        s_over = 0;
    }
    __syncthreads();
    const uint32_t s = t0 + threadIdx.x;
    const uint32_t cap = lbuf.cap;
    uint32_t cnt = 0;
    if (s < N) {
        const SceneView v = S.view(s);  // a staged tile lies in one scene, whose lists are on
        const sim::DeviceParams& dp = *v.dp;
        float R2 = 0.f;
        list_radius2(dp, v.listUpdates, R2);
        const uint32_t key = key_s[s];
        const int reach = neighbour_reach(dp);
        const int side = 2 * reach + 1;
        const int nrows = side * side;  // <= kPlanRows in a staged tile
        const int3 dim = dp.grid.dim;
        int cx, cy, cz;
        decode_key(key - v.cellOffset, dim, cx, cy, cz);
        const int x0 = max(cx - reach, 0);
        const int x1 = min(cx + reach, dim.x - 1);
        const uint32_t* __restrict__ slb = lb + v.cellOffset;
        const float4 pi = pred[s];
        const unsigned long long ix = pk2(pi.x, pi.x), iy = pk2(pi.y, pi.y), iz = pk2(pi.z, pi.z);
        // the interleaved 16-bit list: chunk c at out[c * kListGroup] (2 cap entries of room)
        uint4* out = reinterpret_cast<uint4*>(list16_base(list, cap, s));
        const uint32_t room = 2u * cap;
        // The chunk being filled, as a shift register of eight 16-bit entries:
        // each entry enters at the top of w3 and every earlier one moves down
        // by 16 bits (funnel shifts), so after eight entries the first sits at
        // the bottom of w0.  No branch on the entry's position in the chunk.
        uint32_t w0 = 0u, w1 = 0u, w2 = 0u, w3 = 0u;
        uint32_t shift_of_row = 0;  // stage index of slot k in the current row: k + shift_of_row
        auto shift_in = [&](uint32_t ent) {
            w0 = __funnelshift_r(w0, w1, 16);
            w1 = __funnelshift_r(w1, w2, 16);
            w2 = __funnelshift_r(w2, w3, 16);
            w3 = __funnelshift_r(w3, ent, 16);
        };
        auto emit = [&](uint32_t k) {
            shift_in(k + shift_of_row);
            ++cnt;
            if ((cnt & 7u) == 0u && cnt <= room) out[size_t((cnt >> 3) - 1u) * kListGroup] = make_uint4(w0, w1, w2, w3);
        };
        // Slot range of stencil row r from the lower-bound table ([0, 0) for a
        // row outside the grid).  Row r + 1's range is loaded before row r is
        // walked, so its latency hides behind that walk.
        auto row_range = [&](int r, uint32_t& rb, uint32_t& re) {
            const int z = cz + r / side - reach;
            const int y = cy + r % side - reach;
            rb = re = 0u;
            if (z < 0 || z >= dim.z || y < 0 || y >= dim.y) return;
            const uint32_t row = uint32_t((z * dim.y + y) * dim.x);
            rb = __ldg(slb + row + uint32_t(x0));
            re = __ldg(slb + row + uint32_t(x1) + 1u);
        };
        uint32_t nb, ne;
        row_range(0, nb, ne);
        for (int r = 0; r < nrows; ++r) {
            const uint32_t rb = nb, re = ne;
            if (r + 1 < nrows) row_range(r + 1, nb, ne);
            // the row lies inside the tile's staged range for offset r; the
            // clamp keeps every stage read in bounds regardless
            const uint32_t b = max(rb, P.start[r]);
            const uint32_t e = min(re, P.start[r] + P.len[r]);
            const uint32_t shift = P.base[r] - P.start[r];  // stage index of slot k: k + shift
            shift_of_row = shift;
            // two candidates per round: both loads and tests in flight, then
            // the hits emitted in walk order
            uint32_t k = b;
            for (; k + 1u < e; k += 2u) {
                const float4 pa = sp[k + shift], pb = sp[k + 1u + shift];
                // both candidates' r^2 at once (f32x2: each half is dist2's arithmetic)
                const unsigned long long dx = sub2(ix, pk2(pa.x, pb.x)), dy = sub2(iy, pk2(pa.y, pb.y)),
                                         dz = sub2(iz, pk2(pa.z, pb.z));
                const float2 r2 = upk2(fma2(dz, dz, fma2(dx, dx, mul2(dy, dy))));
                const bool ha = k != s && !(r2.x > R2);
                const bool hb = k + 1u != s && !(r2.y > R2);
                if (ha) emit(k);
                if (hb) emit(k + 1u);
            }
            if (k < e) {
                float rx, ry, rz;
                if (k != s && !(dist2(pi, sp[k + shift], rx, ry, rz) > R2)) emit(k);
            }
        }
        if ((cnt & 7u) && ((cnt + 7u) & ~7u) <= room) {
            // the last, partial chunk: move its entries down to the bottom
            for (uint32_t j = cnt & 7u; j < 8u; ++j) shift_in(0u);
            out[size_t(cnt >> 3) * kListGroup] = make_uint4(w0, w1, w2, w3);
        }
        count[s] = cnt;
    }
    const uint32_t longest = __reduce_max_sync(0xFFFFFFFFu, cnt);
    const uint32_t over = __popc(__ballot_sync(0xFFFFFFFFu, cnt > cap));
    if ((threadIdx.x & 31u) == 0) {
        atomicMax(&s_longest, longest);
        if (over) atomicAdd(&s_over, over);
    }
    __syncthreads();
    if (threadIdx.x == 0 && stats) {
        atomicMax(stats, s_longest);
        if (s_over) atomicAdd(stats + 1, s_over);
    }
}

// lambda of iteration `it` for every slot whose scene runs that iteration,
// into lam[s] and, beside the slot's position, into xl[s] = (x, y, z,
// lambda): the delta pass reads a neighbour's position and lambda with one
// load, and stages its tile by bulk copies of xl.
template <class Scenes, class Sh>
__global__ void __launch_bounds__(Sh::kTile, Sh::kMinSolve) k_lambda(int it, const float4* __restrict__ pred,
                                                  const uint32_t* __restrict__ key_s, const uint32_t* __restrict__ lb,
                                                  Scenes S, uint32_t N, float* __restrict__ lam, ListBufs lbuf,
                                                  uint32_t* __restrict__ err, float4* __restrict__ acc_out,
                                                  float4* __restrict__ xl) {
    extern __shared__ float4 smem[];
    __shared__ TilePlan P;
    float4* sp = smem;
    uint16_t* q16 = reinterpret_cast<uint16_t*>(smem + Sh::kStageMax) + threadIdx.x;
    uint32_t* q32 = reinterpret_cast<uint32_t*>(smem) + threadIdx.x;
    const uint32_t t0 = blockIdx.x * Sh::kTile;
    const uint32_t s = t0 + threadIdx.x;
    const uint32_t sc = s < N ? s : 0u;
    const SceneView v = S.view(sc);
    const sim::DeviceParams dp = *v.dp;  // in registers: the loops below never reload it
    const bool active = s < N && it < v.iters;  // every lane takes part in the warp-wide rounds
    // the slot's own data first: its loads overlap the tile's plan
    const float4 pi = pred[sc];
    const uint32_t cnt = list_count(lbuf, sc);
    const bool staged = plan_and_issue<Sh>(P, key_s, lb, S, lbuf, t0, N, pred, sp);
    const GlobalData g{pred, nullptr, nullptr};
    const bool stageOk = stage_finish<Sh>(P, staged, nullptr, sp, nullptr, err);
    uint32_t n;
    LambdaAcc a;
    if (stageOk && warp_lists_fit(lbuf, active, scene_lists(v, lbuf), cnt, n)) {
        const uint32_t* base = lbuf.list + size_t(sc) * lbuf.cap;
        if (staged)
            a = lambda_queued_acc<kQueue, Sh::kTile>(active, sc, pi,
                                             ListSource<uint16_t>{list16_base(lbuf.list, lbuf.cap, sc), n, 0u, kList16ChunkStride}, dp,
                                             StagedData{sp, nullptr}, q16);
        else
            a = lambda_queued_acc<kQueue, Sh::kTile>(active, sc, pi, ListSource<uint32_t>{base, n, sc}, dp, g, q32);
    } else if (staged) {
        int cx, cy, cz;
        decode_key(key_s[sc] - v.cellOffset, dp.grid.dim, cx, cy, cz);
        if (active)
            a = lambda_of_acc(sc, pi, cx, cy, cz, dp, LbRows{lb + v.cellOffset}, [&](uint32_t k, uint32_t& j) {
                j = k;
                return __ldg(pred + k);
            });
    } else {
        a = lambda_queued_acc<kQueue, Sh::kTile>(active, sc, pi, row_source(key_s, lb, v, sc), dp, g, q32);
    }
    if (!active) return;
    // the neighbour sums, for the adjoint's replay
    if (acc_out) {
        acc_out[2 * size_t(s)] = make_float4(a.density, a.sumGrad2, a.gx, a.gy);
        acc_out[2 * size_t(s) + 1] = make_float4(a.gz, float(a.contrib), __uint_as_float(a.last), 0.f);
    }
    const float l = lambda_finalize(a, dp);
    lam[s] = l;
    xl[s] = make_float4(pi.x, pi.y, pi.z, l);
}

// delta of iteration `it`: neighbours' positions and lambdas from the lambda
// pass's xl, the slot's own prediction from pred (its w is kept) and lambda
// from lam.  The scene's last iteration also applies the post-solve boundary
// (e = 0) and computes v = (x - p)/dt; a scene past its iterations carries
// its prediction through, and a scene without iterations gets boundary and
// velocity in pass 0.  pred_out may be pred itself: a slot reads only its own
// entry of pred, before writing it.
template <class Scenes, class Sh, bool kFast>
__global__ void __launch_bounds__(Sh::kTile, Sh::kMinSolve) k_delta(int it, const float4* __restrict__ xl,
                                                 const float4* pred, const float* __restrict__ lam,
                                                 const uint32_t* __restrict__ key_s, const uint32_t* __restrict__ lb,
                                                 Scenes S, uint32_t N, float4* pred_out,
                                                 const float4* __restrict__ pos_s, float4* __restrict__ vel_s,
                                                 ListBufs lbuf, float4* __restrict__ dsum_out,
                                                 uint32_t* __restrict__ err) {
    extern __shared__ float4 smem[];
    __shared__ TilePlan P;
    float4* sp = smem;
    uint16_t* q16 = reinterpret_cast<uint16_t*>(smem + Sh::kStageMax) + threadIdx.x;
    uint32_t* q32 = reinterpret_cast<uint32_t*>(smem) + threadIdx.x;
    const uint32_t t0 = blockIdx.x * Sh::kTile;
    const uint32_t s = t0 + threadIdx.x;
    const uint32_t sc = s < N ? s : 0u;
    const SceneView v = S.view(sc);
    const sim::DeviceParams dp = *v.dp;  // in registers: the loops below never reload it
    const bool active = s < N && it < v.iters;  // every lane takes part in the warp-wide rounds
    // the slot's own data first: its loads overlap the tile's plan
    const float4 pi = pred[sc];
    const float lam_i = lam[sc];
    // (the many-scene variant keeps the count load late: early, it spills)
    constexpr bool kEarlyCount = std::is_same<Scenes, OneScene>::value;
    const uint32_t cnt = kEarlyCount ? list_count(lbuf, sc) : 0u;
    const bool staged = plan_and_issue<Sh>(P, key_s, lb, S, lbuf, t0, N, xl, sp);
    const float w_q = scorr_wq(dp);
    const PackedData g{xl};
    const bool stageOk = stage_finish<Sh>(P, staged, nullptr, sp, nullptr, err);
    uint32_t n;
    float3 d = make_float3(0.f, 0.f, 0.f);
    if (stageOk &&
        warp_lists_fit(lbuf, active, scene_lists(v, lbuf), kEarlyCount ? cnt : list_count(lbuf, sc), n)) {
        const uint32_t* base = lbuf.list + size_t(sc) * lbuf.cap;
        if (staged)
            d = delta_queued_sum<kQueue, Sh::kTile, kFast>(active, sc, pi, lam_i,
                                            ListSource<uint16_t>{list16_base(lbuf.list, lbuf.cap, sc), n, 0u, kList16ChunkStride}, dp,
                                            w_q, StagedData{sp, nullptr}, q16);
        else
            d = delta_queued_sum<kQueue, Sh::kTile, kFast>(active, sc, pi, lam_i, ListSource<uint32_t>{base, n, sc}, dp, w_q, g,
                                            q32);
    } else if (staged) {
        int cx, cy, cz;
        decode_key(key_s[sc] - v.cellOffset, dp.grid.dim, cx, cy, cz);
        if (active)
            d = delta_of_sum<kFast>(sc, pi, lam_i, cx, cy, cz, dp, w_q, LbRows{lb + v.cellOffset},
                         [&](uint32_t k, uint32_t& j, float& lj) {
                             j = k;
                             const float4 pk = __ldg(xl + k);
                             lj = pk.w;
                             return pk;
                         });
    } else {
        d = delta_queued_sum<kQueue, Sh::kTile, kFast>(active, sc, pi, lam_i, row_source(key_s, lb, v, sc), dp, w_q, g, q32);
    }
    // the neighbour sum, for the adjoint's replay (which needs the displacement
    // before the clamp)
    if (dsum_out && active) dsum_out[s] = make_float4(d.x, d.y, d.z, 0.f);
    if (active) d = delta_finalize(d, dp);
    if (s >= N) return;
    const bool last = active ? it == v.iters - 1 : (v.iters <= 0 && it == 0);
    float4 x = active ? make_float4(add_(pi.x, d.x), add_(pi.y, d.y), add_(pi.z, d.z), pi.w) : pi;
    if (last) {
        // Boundary(e=0) after the solve loop (sim/phases.cpp:94); its velocity
        // half is overwritten by the velocity phase, so only x is clamped.
        float4 vdummy = make_float4(0.f, 0.f, 0.f, 0.f);
        boundary_apply(x, vdummy, dp.grid, 0.0f);
        // PhaseVelocity (sim/phases.cpp:102-105): v = (x - p) * (1/dt).
        const float inv_dt = div_(1.0f, dp.dt);
        const float4 p = pos_s[s];
        vel_s[s] = make_float4(mul_(sub_(x.x, p.x), inv_dt), mul_(sub_(x.y, p.y), inv_dt),
                               mul_(sub_(x.z, p.z), inv_dt), 0.0f);
    }
    pred_out[s] = x;
}

// solverIters == 0: the boundary and velocity phases on the prediction.
__global__ void __launch_bounds__(kBS) k_finalize_no_iters(float4* __restrict__ pred, const float4* __restrict__ pos_s,
                                                           const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                           float4* __restrict__ vel_s) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    float4 x = pred[s];
    float4 vdummy = make_float4(0.f, 0.f, 0.f, 0.f);
    boundary_apply(x, vdummy, dpp->grid, 0.0f);
    const float inv_dt = div_(1.0f, dpp->dt);
    const float4 p = pos_s[s];
    vel_s[s] = make_float4(mul_(sub_(x.x, p.x), inv_dt), mul_(sub_(x.y, p.y), inv_dt), mul_(sub_(x.z, p.z), inv_dt),
                           0.0f);
    pred[s] = x;
}

// XSPH (Jacobi, where the scene configures it), boundary(e), scatter to ids.
template <class Scenes, bool kXsph, class Sh>
__global__ void __launch_bounds__(Sh::kTile, Sh::kMinCommit) k_commit(const float4* __restrict__ pred, const float4* __restrict__ vel_s,
                                                  const uint32_t* __restrict__ key_s, const uint32_t* __restrict__ lb,
                                                  const uint32_t* __restrict__ perm, Scenes S, uint32_t N,
                                                  float4* __restrict__ pos, float4* __restrict__ vel, ListBufs lbuf,
                                                  uint32_t* __restrict__ err) {
    extern __shared__ float4 smem[];
    __shared__ TilePlan P;
    const uint32_t t0 = blockIdx.x * Sh::kTile;
    const uint32_t s = t0 + threadIdx.x;
    const uint32_t sc = s < N ? s : 0u;
    const SceneView v = S.view(sc);
    const sim::DeviceParams dp = *v.dp;  // in registers: the loops below never reload it
    float4 x = pred[sc];
    float4 vv = vel_s[sc];
    if (kXsph) {
        float4* sp = smem;
        float2* sv = reinterpret_cast<float2*>(smem + Sh::kStageMax);
        const bool xs = s < N && dp.xsph_c > 0.f;  // every lane takes part in the warp-wide rounds
        const uint32_t cnt = list_count(lbuf, sc);
        const bool staged = plan_and_issue<Sh>(P, key_s, lb, S, lbuf, t0, N, pred, sp);
        const bool stageOk = stage_finish<Sh>(P, staged, vel_s, sp, sv, err);
        // Queue of the queued walks: the stage area, free in tiles that are
        // not staged.  In a staged tile a warp whose lists overflowed walks
        // the stencil without a queue.
        uint32_t* q = reinterpret_cast<uint32_t*>(smem) + threadIdx.x;
        const GlobalData g{pred, nullptr, vel_s};
        uint32_t n;
        float4 vx = vv;
        if (stageOk && warp_lists_fit(lbuf, xs, scene_lists(v, lbuf), cnt, n)) {
            const uint32_t* base = lbuf.list + size_t(sc) * lbuf.cap;
            if (staged)
                vx = xsph_list_inline(xs, x, vv,
                                      ListSource<uint16_t>{list16_base(lbuf.list, lbuf.cap, sc), n, 0u, kList16ChunkStride}, dp,
                                      StagedData{sp, sv});
            else
                vx = xsph_queued<kQueue, Sh::kTile>(xs, sc, x, vv, ListSource<uint32_t>{base, n, sc}, dp, g, q);
        } else if (staged) {
            int cx, cy, cz;
            decode_key(key_s[sc] - v.cellOffset, dp.grid.dim, cx, cy, cz);
            if (xs)
                vx = xsph_of(sc, x, vv, cx, cy, cz, dp, LbRows{lb + v.cellOffset},
                             [&](uint32_t k, uint32_t& j, float4& vj) {
                                 j = k;
                                 vj = __ldg(vel_s + k);
                                 return __ldg(pred + k);
                             });
        } else {
            vx = xsph_queued<kQueue, Sh::kTile>(xs, sc, x, vv, row_source(key_s, lb, v, sc), dp, g, q);
        }
        if (xs) vv = vx;
    }
    if (s < N) boundary_apply(x, vv, dp.grid, dp.boundaryRestitution);
    // a NaN / Inf in the committed state is reported through the error word
    const bool bad = s < N && !(isfinite(x.x) && isfinite(x.y) && isfinite(x.z) && isfinite(vv.x) &&
                                isfinite(vv.y) && isfinite(vv.z));
    if (__any_sync(0xFFFFFFFFu, bad) && (threadIdx.x & 31u) == 0 && err) atomicOr(err, kErrNonFiniteBit);
    if (s >= N) return;
    const uint32_t i = perm[s];
    pos[i] = x;
    vel[i] = vv;
}

__global__ void k_scatter_lambda(const float* __restrict__ lam_s, const uint32_t* __restrict__ perm, uint32_t N,
                                 float* __restrict__ out) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    out[perm[s]] = lam_s[s];
}

// ---------------------------------------------------------------- stats
__global__ void __launch_bounds__(kBS) k_position_keys(const float4* __restrict__ pos,
                                                       const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                       uint32_t* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    keys[i] = cell_key(pos[i], dpp->grid);
}

__global__ void __launch_bounds__(kBS) k_gather_positions(const uint32_t* __restrict__ perm,
                                                          const float4* __restrict__ pos, uint32_t N,
                                                          float4* __restrict__ out) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    out[s] = pos[perm[s]];
}

// Per-block partial sums of |C|, max|C|, max(C,0), neighbour count over a
// fixed slot range, reduced in a fixed tree order (deterministic).
__global__ void __launch_bounds__(kBS) k_density_partials(const float4* __restrict__ xs,
                                                          const uint32_t* __restrict__ key_s,
                                                          const uint32_t* __restrict__ lb,
                                                          const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                          uint32_t perBlock, double* __restrict__ partials) {
    const sim::DeviceParams& dp = *dpp;
    const sim::KernelCoeffs& kc = dp.kernel;
    double a = 0, m = 0, pc = 0, nb = 0;
    const uint32_t beg = blockIdx.x * perBlock;
    const uint32_t end = min(N, beg + perBlock);
    for (uint32_t s = beg + threadIdx.x; s < end; s += blockDim.x) {
        int cx, cy, cz;
        decode_key(key_s[s], dp.grid.dim, cx, cy, cz);
        const float4 pi = xs[s];
        float rho = 0.f;
        int cnt = 0;
        walk_neighbours(cx, cy, cz, neighbour_reach(dp), dp.grid.dim, LbRows{lb}, [&](uint32_t k) -> bool {
            if (k == s) return true;
            const float4 pj = __ldg(xs + k);
            const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            const float r2 = rx * rx + ry * ry + rz * rz;
            if (r2 > kc.h2) return true;
            const float hr2 = kc.h2 - r2;
            rho += dp.particleMass * kc.poly6 * hr2 * hr2 * hr2;
            ++cnt;
            return true;
        });
        const double C = (dp.restDensity > 0.f) ? double(rho) / double(dp.restDensity) - 1.0 : 0.0;
        a += fabs(C);
        m = fmax(m, fabs(C));
        pc += C > 0 ? C : 0.0;
        nb += cnt;
    }
    __shared__ double sh[4][kBS];
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = m;
    sh[2][threadIdx.x] = pc;
    sh[3][threadIdx.x] = nb;
    __syncthreads();
    for (int w = kBS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
            sh[1][threadIdx.x] = fmax(sh[1][threadIdx.x], sh[1][threadIdx.x + w]);
            sh[2][threadIdx.x] += sh[2][threadIdx.x + w];
            sh[3][threadIdx.x] += sh[3][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[4 * blockIdx.x + 0] = sh[0][0];
        partials[4 * blockIdx.x + 1] = sh[1][0];
        partials[4 * blockIdx.x + 2] = sh[2][0];
        partials[4 * blockIdx.x + 3] = sh[3][0];
    }
}

__global__ void k_density_final(const double* __restrict__ partials, unsigned nblocks, uint32_t N,
                                 double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0, m = 0, pc = 0, nb = 0;
    for (unsigned b = 0; b < nblocks; ++b) {
        a += partials[4 * b + 0];
        m = fmax(m, partials[4 * b + 1]);
        pc += partials[4 * b + 2];
        nb += partials[4 * b + 3];
    }
    const double n = N ? double(N) : 1.0;
    out[0] = a / n;
    out[1] = m;
    out[2] = pc / n;
    out[3] = nb / n;
}

}  // namespace

cudaError_t fused_predict_keys(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    if (sh.N == 0) return cudaSuccess;
    k_predict_keys<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.pos, b.vel, b.dp, sh.N, b.keys);
    return cudaGetLastError();
}

cudaError_t fused_sort(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    return sort_pairs(b.sort_temp, b.sort_bytes, b.keys, b.key_s, nullptr, b.perm, sh.N, sh.key_bits, s, b.err);
}

cudaError_t fused_gather_and_tables(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    // The gather, the lower-bound table and the compact table read only the
    // sorted keys and permutation, and write disjoint buffers: with the fork
    // resources they run side by side (each is a few small, latency-bound
    // kernels), joined back on s.
    const bool fork = b.fork_streams[0] && b.fork_streams[1] && b.fork_events[0] && b.fork_events[1] &&
                      b.fork_events[2];
    cudaStream_t s_lb = s, s_cp = s;
    cudaError_t e;
    if (fork) {
        if ((e = cudaEventRecord(b.fork_events[0], s)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(b.fork_streams[0], b.fork_events[0], 0)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(b.fork_streams[1], b.fork_events[0], 0)) != cudaSuccess)
            return e;
        s_lb = b.fork_streams[0];
        s_cp = b.fork_streams[1];
    }
    if (sh.N > 0) k_gather<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.perm, b.pos, b.vel, b.dp, sh.N, b.pred_a, b.pos_s);
    e = launch_cell_lb(b.lb, b.key_s, sh.N, sh.numCells, s_lb);
    if (e == cudaSuccess && sh.hashed)
        e = launch_compact(b.compact_temp, b.compact_bytes, b.uk, b.off, b.count, nullptr, b.key_s, sh.N, s_cp, b.err);
    if (fork) {
        // join even after a failed launch, so that a capture stays well formed
        const cudaError_t j = (cudaEventRecord(b.fork_events[1], s_lb) == cudaSuccess &&
                               cudaEventRecord(b.fork_events[2], s_cp) == cudaSuccess &&
                               cudaStreamWaitEvent(s, b.fork_events[1], 0) == cudaSuccess &&
                               cudaStreamWaitEvent(s, b.fork_events[2], 0) == cudaSuccess)
                                  ? cudaSuccess
                                  : cudaErrorUnknown;
        if (e == cudaSuccess) e = j;
    }
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

int list_span_for(const sim::SimParams& p) {
    if (!p.pbf.enable_disp_clamp || p.solverIters <= 0) return 0;
    const float md = std::fabs(p.pbf.disp_clamp_max_h);
    if (!(md < 1.0f)) return 0;  // NaN, or updates move particles by h or more
    const int iters = p.solverIters;
    // One list for the whole step while its radius h + 2 * iters * md stays
    // within 1.5 h.
    if (2.0f * float(iters) * md <= 0.5f) return iters;
    // Otherwise a list per span of iterations whose lambda / delta passes read
    // at most span - 1 updates after the build (radius <= 1.25 h); the commit
    // then walks the stencil.
    const int span = int(0.125f / md) + 1;
    return span >= 2 ? std::min(span, iters - 1) : 0;
}

namespace {

bool lists_on(const FusedBufs& b, const FusedShape& sh) {
    return sh.list_span > 0 && b.nbr_cap > 0 && b.nbr_list && b.nbr_count && sh.iters > 0;
}

// Position updates the list serving iteration `it` (it == iters: the commit)
// must cover, or -1 when that pass walks the stencil.
//   * One list (span >= iters): built from the prediction p0, which lies in
//     the box; the passes read p0 .. p_{iters-1} and the commit reads
//     p_iters = P(p0 + D), P the projection onto the box, and since
//     |P(p0 + D) - p0| = |P(p0 + D) - P(p0)| <= |D|, every pass is within
//     iters clamped updates of p0.
//   * A list per span: a span's lambda / delta passes read the predictions
//     p_start .. p_{start+span-1}, no boundary in between, so span - 1
//     updates.  The commit is not covered: p_start may lie outside the box
//     and the final projection may move it further than the remaining
//     updates.
int list_updates(const FusedShape& sh, int it) {
    if (sh.list_span >= sh.iters) return sh.iters;
    return it >= sh.iters ? -1 : sh.list_span - 1;
}

ListBufs list_bufs(const FusedBufs& b, const FusedShape& sh) {
    if (!lists_on(b, sh)) return ListBufs{nullptr, nullptr, 0u, 0, nullptr};
    return ListBufs{b.nbr_list, b.nbr_count, b.nbr_cap, b.nbr_staging ? 1 : 0, b.tile_plans};
}

OneScene one_scene(const FusedBufs& b, const FusedShape& sh, int it) {
    return OneScene{b.dp, sh.iters, lists_on(b, sh) ? list_updates(sh, it) : -1};
}

}  // namespace

int fused_list_builds(const FusedShape& sh) {
    if (sh.list_span <= 0 || sh.iters <= 0) return 0;
    return (sh.iters + sh.list_span - 1) / sh.list_span;
}

namespace {

// Calls f with the tile shape `id` names (an unknown id takes shape 0).
template <class F>
cudaError_t with_tile_shape(int id, F&& f) {
    switch (id) {
    case 1: return f(TileShape1{});
    case 2: return f(TileShape2{});
    case 3: return f(TileShape3{});
    default: return f(TileShape0{});
    }
}

// Calls f with std::integral_constant<bool, fast> for the arithmetic mode.
template <class F>
cudaError_t with_math(bool fast, F&& f) {
    return fast ? f(std::true_type{}) : f(std::false_type{});
}

template <class Sh>
cudaError_t prepare_solve() {
    const int solve = int(Sh::kSolveSmem);
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_lambda<OneScene, Sh>, a, solve)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_lambda<ManyScenes, Sh>, a, solve)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_delta<OneScene, Sh, false>, a, solve)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_delta<ManyScenes, Sh, false>, a, solve)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_delta<OneScene, Sh, true>, a, solve)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_delta<ManyScenes, Sh, true>, a, solve)) != cudaSuccess)
        return e;
    return cudaSuccess;
}

template <class Sh>
cudaError_t prepare_shape() {
    const int commit = int(Sh::kCommitSmem), stage = int(Sh::kStageBytes);
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e;
    if ((e = prepare_solve<Sh>()) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_build_lists_tiled<OneScene, Sh>, a, stage)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_build_lists_tiled<ManyScenes, Sh>, a, stage)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_commit<OneScene, true, Sh>, a, commit)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_commit<OneScene, false, Sh>, a, commit)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_commit<ManyScenes, true, Sh>, a, commit)) != cudaSuccess)
        return e;
    return cudaSuccess;
}

}  // namespace

int fused_tile_shape_count() { return kTileShapeCount; }

size_t fused_tile_plan_bytes(uint32_t capacity) {
    int smallest = 1 << 30;
    for (int id = 0; id < kTileShapeCount; ++id) {
        int tile = 0, stage = 0;
        fused_tile_shape_info(id, tile, stage);
        smallest = std::min(smallest, tile);
    }
    const size_t tiles = (size_t(capacity) + size_t(smallest) - 1) / size_t(smallest) + 1;
    return tiles * kPlanStride * sizeof(uint4);
}

bool fused_tile_shape_info(int id, int& tile, int& stage) {
    if (id < 0 || id >= kTileShapeCount) return false;
    with_tile_shape(id, [&](auto shape) {
        using Sh = decltype(shape);
        tile = Sh::kTile;
        stage = Sh::kStageMax;
        return cudaSuccess;
    });
    return true;
}

// Opts the list passes of every tile shape into their dynamic shared memory
// (above the 48 KB default); once per process and device, before the first
// launch or capture.
cudaError_t fused_prepare_kernels() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev]) return cudaSuccess;
    if ((e = prepare_shape<TileShape0>()) != cudaSuccess || (e = prepare_shape<TileShape1>()) != cudaSuccess ||
        (e = prepare_shape<TileShape2>()) != cudaSuccess || (e = prepare_shape<TileShape3>()) != cudaSuccess)
        return e;
    done[dev] = true;
    return cudaSuccess;
}

cudaError_t fused_build_lists(const FusedBufs& b, const FusedShape& sh, int it, cudaStream_t s) {
    if (sh.N == 0 || !lists_on(b, sh) || it < 0 || it >= sh.iters || it % sh.list_span != 0) return cudaErrorNotReady;
    const cudaError_t pe = fused_prepare_kernels();
    if (pe != cudaSuccess) return pe;
    const float4* cur = b.pred_a;
    return with_tile_shape(sh.tile, [&](auto shape) {
        using Sh = decltype(shape);
        k_build_lists_tiled<OneScene, Sh><<<blocks_for(sh.N, Sh::kTile), Sh::kTile, Sh::kStageBytes, s>>>(
            cur, b.key_s, b.lb, one_scene(b, sh, it), sh.N, list_bufs(b, sh), b.nbr_list, b.nbr_count, b.nbr_stats,
            b.err);
        return cudaGetLastError();
    });
}

cudaError_t fused_solve_phase(const FusedBufs& b, const FusedShape& sh, int it, int which, cudaStream_t s) {
    if (sh.N == 0 || it < 0 || it >= sh.iters) return cudaSuccess;
    cudaError_t e = fused_prepare_kernels();
    if (e != cudaSuccess) return e;
    // lambda reads the prediction in pred_a and writes (x, y, z, lambda) to
    // pred_b; delta reads pred_b and writes the next prediction to pred_next
    // (default: over pred_a)
    float4* cur = b.pred_a;
    float4* xl = b.pred_b;
    float4* nxt = b.pred_next ? b.pred_next : b.pred_a;
    const OneScene sc = one_scene(b, sh, it);
    return with_tile_shape(sh.tile, [&](auto shape) {
        using Sh = decltype(shape);
        return with_math(sh.fast, [&](auto fast) {
            constexpr bool kFast = decltype(fast)::value;
            const unsigned g = blocks_for(sh.N, Sh::kTile);
            if (which == 0)
                k_lambda<OneScene, Sh><<<g, Sh::kTile, Sh::kSolveSmem, s>>>(
                    it, cur, b.key_s, b.lb, sc, sh.N, b.lam_s, list_bufs(b, sh), b.err, b.lambda_acc, xl);
            else
                k_delta<OneScene, Sh, kFast><<<g, Sh::kTile, Sh::kSolveSmem, s>>>(
                    it, xl, cur, b.lam_s, b.key_s, b.lb, sc, sh.N, nxt, b.pos_s, b.vel_s, list_bufs(b, sh),
                    b.delta_sum, b.err);
            return cudaGetLastError();
        });
    });
}

cudaError_t fused_solve(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    if (sh.N == 0) return cudaSuccess;
    for (int it = 0; it < sh.iters; ++it) {
        cudaError_t e = fused_build_lists(b, sh, it, s);
        if (e != cudaSuccess && e != cudaErrorNotReady) return e;
        if ((e = fused_solve_phase(b, sh, it, 0, s)) != cudaSuccess) return e;
        if ((e = fused_solve_phase(b, sh, it, 1, s)) != cudaSuccess) return e;
    }
    if (sh.iters <= 0)
        k_finalize_no_iters<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.pred_a, b.pos_s, b.dp, sh.N, b.vel_s);
    return cudaGetLastError();
}

cudaError_t fused_commit(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    if (sh.N == 0) return cudaSuccess;
    cudaError_t e = fused_prepare_kernels();
    if (e != cudaSuccess) return e;
    const float4* x = fused_final_pred(b, sh);
    const OneScene sc = one_scene(b, sh, sh.iters);
    const ListBufs lb = list_bufs(b, sh);
    return with_tile_shape(sh.tile, [&](auto shape) {
        using Sh = decltype(shape);
        const unsigned g = blocks_for(sh.N, Sh::kTile);
        if (sh.xsph)
            k_commit<OneScene, true, Sh><<<g, Sh::kTile, Sh::kCommitSmem, s>>>(x, b.vel_s, b.key_s, b.lb, b.perm, sc,
                                                                                sh.N, b.pos, b.vel, lb, b.err);
        else
            k_commit<OneScene, false, Sh><<<g, Sh::kTile, Sh::kCommitSmem, s>>>(x, b.vel_s, b.key_s, b.lb, b.perm, sc,
                                                                                 sh.N, b.pos, b.vel, lb, b.err);
        return cudaGetLastError();
    });
}

// ------------------------------------------------------------ many scenes
cudaError_t multi_build_lists(const MultiBufs& m, cudaStream_t s) {
    if (m.N == 0 || m.nbr_cap == 0) return cudaSuccess;
    const cudaError_t pe = fused_prepare_kernels();
    if (pe != cudaSuccess) return pe;
    const ListBufs lb{m.nbr_list, m.nbr_count, m.nbr_cap, 1, m.tile_plans};
    return with_tile_shape(m.tile, [&](auto shape) {
        using Sh = decltype(shape);
        k_build_lists_tiled<ManyScenes, Sh><<<blocks_for(m.N, Sh::kTile), Sh::kTile, Sh::kStageBytes, s>>>(
            m.pred_a, m.key_s, m.lb, ManyScenes{m.scenes, m.sceneOfSlot}, m.N, lb, m.nbr_list, m.nbr_count,
            m.nbr_stats, m.err);
        return cudaGetLastError();
    });
}

cudaError_t multi_solve_phase(const MultiBufs& m, int it, int which, cudaStream_t s) {
    if (m.N == 0) return cudaSuccess;
    cudaError_t e = fused_prepare_kernels();
    if (e != cudaSuccess) return e;
    // as fused_solve_phase: the prediction stays in pred_a, pred_b holds (x, y, z, lambda)
    float4* cur = m.pred_a;
    float4* xl = m.pred_b;
    const ManyScenes sc{m.scenes, m.sceneOfSlot};
    const ListBufs lb{m.nbr_list, m.nbr_count, m.nbr_cap, 1, m.tile_plans};
    return with_tile_shape(m.tile, [&](auto shape) {
        using Sh = decltype(shape);
        return with_math(m.fast, [&](auto fast) {
            constexpr bool kFast = decltype(fast)::value;
            const unsigned g = blocks_for(m.N, Sh::kTile);
            if (which == 0)
                k_lambda<ManyScenes, Sh><<<g, Sh::kTile, Sh::kSolveSmem, s>>>(it, cur, m.key_s, m.lb, sc, m.N,
                                                                                    m.lam_s, lb, m.err, nullptr, xl);
            else
                k_delta<ManyScenes, Sh, kFast><<<g, Sh::kTile, Sh::kSolveSmem, s>>>(
                    it, xl, cur, m.lam_s, m.key_s, m.lb, sc, m.N, cur, m.pos_s, m.vel_s, lb, nullptr, m.err);
            return cudaGetLastError();
        });
    });
}

cudaError_t multi_commit(const MultiBufs& m, const float4* final_pred, cudaStream_t s) {
    if (m.N == 0) return cudaSuccess;
    cudaError_t e = fused_prepare_kernels();
    if (e != cudaSuccess) return e;
    const ListBufs lb{m.nbr_list, m.nbr_count, m.nbr_cap, 1, m.tile_plans};
    return with_tile_shape(m.tile, [&](auto shape) {
        using Sh = decltype(shape);
        k_commit<ManyScenes, true, Sh><<<blocks_for(m.N, Sh::kTile), Sh::kTile, Sh::kCommitSmem, s>>>(
            final_pred, m.vel_s, m.key_s, m.lb, m.perm, ManyScenes{m.scenes, m.sceneOfSlot}, m.N, m.pos, m.vel, lb,
            m.err);
        return cudaGetLastError();
    });
}

// Failure path of the staging wait: one block arms its barrier for 16 bytes
// that no copy delivers, so the bounded wait gives up, records
// kErrStageTimeoutBit in err[0] and returns (no copy is in flight).
__global__ void k_selftest_stage_wait(uint32_t limit, uint32_t* __restrict__ err) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_arrive_expect_tx(&bar, 16u);
    }
    __syncthreads();
    if (!mbar_wait_bounded(&bar, 0u, limit) && threadIdx.x == 0) atomicOr(err, kErrStageTimeoutBit);
}

cudaError_t fused_selftest_stage_wait(uint32_t spin_limit, uint32_t* d_err, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    k_selftest_stage_wait<<<1, 32, 0, s>>>(spin_limit, d_err);
    return cudaGetLastError();
}

cudaError_t fused_scatter_lambda(const FusedBufs& b, const FusedShape& sh, float* lambda_by_id, cudaStream_t s) {
    if (sh.N == 0) return cudaSuccess;
    k_scatter_lambda<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.lam_s, b.perm, sh.N, lambda_by_id);
    return cudaGetLastError();
}

cudaError_t fused_density_stats(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    if (sh.N == 0) return cudaMemsetAsync(b.stats_out, 0, 4 * sizeof(double), s);
    // Fresh grid over the committed positions (keys -> sort -> lb), using the
    // step's sorted buffers as scratch.
    k_position_keys<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.pos, b.dp, sh.N, b.keys);
    cudaError_t e = sort_pairs(b.sort_temp, b.sort_bytes, b.keys, b.key_s, nullptr, b.perm, sh.N, sh.key_bits, s, b.err);
    if (e != cudaSuccess) return e;
    k_gather_positions<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.perm, b.pos, sh.N, b.pred_b);
    e = launch_cell_lb(b.lb, b.key_s, sh.N, sh.numCells, s);
    if (e != cudaSuccess) return e;
    unsigned nb = blocks_for(sh.N, 1024u);
    if (nb > kStatsMaxBlocks) nb = kStatsMaxBlocks;
    const uint32_t perBlock = (sh.N + nb - 1) / nb;
    k_density_partials<<<nb, kBS, 0, s>>>(b.pred_b, b.key_s, b.lb, b.dp, sh.N, perBlock, b.stats_partials);
    k_density_final<<<1, 32, 0, s>>>(b.stats_partials, nb, sh.N, b.stats_out);
    return cudaGetLastError();
}

}  // namespace pbf
