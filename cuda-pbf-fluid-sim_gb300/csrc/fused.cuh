// fused.cuh - the fused GB300 step (host launch helpers).
//
// Data layout in HBM for one scene of N particles:
//   pos, vel        float4[N]   committed state, original particle order
//   keys            u32[N]      cell key of each particle's prediction (id order)
//   key_s, perm     u32[N]      sorted keys and sorted->original ids
//   pred_a          float4[N]   predicted positions in cell order (each solver
//                               iteration's delta pass updates them in place)
//   pred_b          float4[N]   (x, y, z, lambda) of the current iteration in
//                               cell order (lambda pass -> delta pass)
//   pos_s, vel_s    float4[N]   step-start positions / velocities in cell order
//   lam_s           f32[N]      lambda in cell order
//   lb              u32[numCells+1]  dense lower-bound table
//   uk, off, count  compact table (hashed strategy)
// Every neighbour pass reads positions in cell order, so a warp's candidate
// loads fall in a few consecutive cache lines instead of N random gathers.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pbf/parameters.h"

namespace pbf {

struct FusedBufs {
    float4* pos;
    float4* vel;
    uint32_t* keys;
    uint32_t* key_s;
    uint32_t* perm;
    float4* pred_a;
    float4* pred_b;
    // Optional (null: pred_a): where the delta passes write the next
    // prediction (the adjoint's replay keeps every iteration's).
    float4* pred_next;
    // Optional (null: each list pass plans its tiles): fused_tile_plan_bytes
    // of scratch where the list build stores the step's tile plans for the
    // passes after it.
    uint4* tile_plans;
    // Optional (any null: one stream): side streams and events on which
    // fused_gather_and_tables runs the lower-bound and compact tables beside
    // the gather, joined back on its stream before it returns.
    cudaStream_t fork_streams[2];
    cudaEvent_t fork_events[3];
    // Optional (null: not written): the delta pass's neighbour sum per sorted
    // slot, before the displacement clamp (the adjoint's replay records it).
    float4* delta_sum;
    // Optional: the lambda pass's neighbour sums per sorted slot, two float4
    // each: (density, sum |grad|^2, grad x, grad y), (grad z, contributions,
    // bits of the last neighbour's index, 0).
    float4* lambda_acc;
    float4* pos_s;
    float4* vel_s;
    float* lam_s;
    uint32_t* lb;
    uint32_t* uk;
    uint32_t* off;
    uint32_t* count;
    void* sort_temp;
    size_t sort_bytes;
    void* compact_temp;
    size_t compact_bytes;
    const sim::DeviceParams* dp;  // device-resident parameter block
    uint32_t* err;                // device error word
    double* stats_partials;       // device, >= kStatsMaxBlocks * 4 doubles
    double* stats_out;            // device, 4 doubles
    // Neighbour lists (cell order): particle s owns entries
    // nbr_list[s * nbr_cap, (s + 1) * nbr_cap); nbr_count[s] is its length
    // (> nbr_cap: overflowed, the particle's warp walks the stencil instead).
    // nbr_stats[0] = longest list built, nbr_stats[1] = overflowed lists
    // (both accumulate until the host clears them).
    uint32_t* nbr_list;
    uint32_t* nbr_count;
    uint32_t* nbr_stats;
    uint32_t nbr_cap;  // entries per particle, a multiple of 8; 0 = no lists
    // false: every list holds 32-bit sorted slots (no tile is staged), for
    // lists that are read outside the list passes (the adjoint)
    bool nbr_staging = true;
};

struct FusedShape {
    uint32_t N;
    uint32_t numCells;
    int key_bits;
    int iters;
    bool hashed;
    bool xsph;
    // Solver iterations one neighbour list covers (lists are built before
    // lambda of iterations 0, span, 2*span, ...); 0 = every pass walks the
    // stencil.
    int list_span;
    // Tile shape of the list passes (0 .. fused_tile_shape_count() - 1).
    int tile;
    // Arithmetic of the delta pass: false = exact (bit-identical to the
    // reference kernels), true = fast (s_corr power from error-free products
    // instead of powf; within the 1e-5 bars).
    bool fast;
};

// Tile shapes the list passes are compiled for: slots per tile (threads per
// CTA) and slots a tile's stage holds.  Results do not depend on the shape.
constexpr int kTileShapeCount = 4;
int fused_tile_shape_count();
bool fused_tile_shape_info(int id, int& tile, int& stage);
// The autotuner's choice among measured step times: the fastest shape, but
// the current one is kept unless the fastest beats it by kTileShapeMargin (a
// few steps of one state do not rank shapes that close).
constexpr float kTileShapeMargin = 0.02f;
inline int pick_tile_shape(const float* ms, int n, int current) {
    int best = (current >= 0 && current < n) ? current : 0;
    for (int i = 0; i < n; ++i)
        if (ms[i] < ms[best]) best = i;
    if (best != current && current >= 0 && current < n && !(ms[best] < ms[current] * (1.0f - kTileShapeMargin)))
        return current;
    return best;
}

// Iterations a list may cover for these parameters: the list radius grows by
// 2 * disp_clamp_max_h * h per covered position update; lists are rebuilt
// once it would pass 1.25 h.  0 when the displacement clamp is off (no bound
// on how far particles move, so no list is valid).
int list_span_for(const sim::SimParams& p);

constexpr unsigned kStatsMaxBlocks = 1024;

// One-time per-device kernel setup (shared-memory opt-in of the list passes);
// the launchers call it too, but it must first run outside stream capture.
cudaError_t fused_prepare_kernels();

// Phase launchers of the fused step (each one graph-capturable).
cudaError_t fused_predict_keys(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);
cudaError_t fused_sort(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);
cudaError_t fused_gather_and_tables(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);
cudaError_t fused_solve(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);
cudaError_t fused_commit(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);
// One kernel of the solve loop: iteration `it`, which = 0 (lambda) or 1
// (delta).  fused_solve == all of them in order, each iteration's lambda
// preceded by fused_build_lists.
cudaError_t fused_solve_phase(const FusedBufs& b, const FusedShape& sh, int it, int which, cudaStream_t s);
// Builds the neighbour lists if iteration `it` starts a list span; returns
// cudaErrorNotReady (and launches nothing) when it does not.
cudaError_t fused_build_lists(const FusedBufs& b, const FusedShape& sh, int it, cudaStream_t s);
// Bytes of FusedBufs::tile_plans for up to `capacity` particles (every tile
// shape).
size_t fused_tile_plan_bytes(uint32_t capacity);
// Number of list builds per step.
int fused_list_builds(const FusedShape& sh);
// Sorted buffer holding the solved prediction after fused_solve.
inline float4* fused_final_pred(const FusedBufs& b, const FusedShape&) { return b.pred_a; }

// ------------------------------------------------------------ many scenes
// One scene of a batch: its parameters, its first cell in the batch's global
// cell numbering, its solver iterations and the position updates its
// neighbour lists cover (-1: the scene walks the stencil).
struct SceneInfo {
    sim::DeviceParams dp;
    uint32_t cellOffset;
    int iters;
    int listUpdates;
    int pad;
};

// Buffers of a batch of scenes (sorted slots over all scenes).
struct MultiBufs {
    uint32_t N;
    const SceneInfo* scenes;
    const uint32_t* sceneOfSlot;
    float4 *pos, *vel, *pred_a, *pred_b, *pos_s, *vel_s;
    float* lam_s;
    const uint32_t *key_s, *perm, *lb;
    uint32_t *nbr_list, *nbr_count, *nbr_stats;
    uint32_t nbr_cap;  // 0: no lists
    uint4* tile_plans; // as FusedBufs::tile_plans
    uint32_t* err;     // device error word (kErr* bits)
    int tile;          // tile shape of the list passes
    bool fast;         // arithmetic of the delta pass (FusedShape::fast)
};

// The list passes of a batch: lists built once from the prediction (for the
// scenes whose listUpdates >= 0), lambda / delta of iteration `it` for every
// scene that runs it (scenes past their iterations carry the prediction
// through), and XSPH + boundary + scatter.
cudaError_t multi_build_lists(const MultiBufs& m, cudaStream_t s);
cudaError_t multi_solve_phase(const MultiBufs& m, int it, int which, cudaStream_t s);
cudaError_t multi_commit(const MultiBufs& m, const float4* final_pred, cudaStream_t s);

// Density statistics of the committed state (fresh grid; uses pred_b/pos_s
// as scratch).  Writes 4 doubles to b.stats_out.
cudaError_t fused_density_stats(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);

// Failure-path self-test of the staging barrier's bounded wait (see
// pbf_selftest_stage_wait); d_err receives the error word.
cudaError_t fused_selftest_stage_wait(uint32_t spin_limit, uint32_t* d_err, cudaStream_t s);

// lambda (by original id) of the last iteration, for inspection.
cudaError_t fused_scatter_lambda(const FusedBufs& b, const FusedShape& sh, float* lambda_by_id, cudaStream_t s);

}  // namespace pbf
