// fused.cuh - the fused GB300 step (host launch helpers).
//
// Data layout in HBM for one scene of N particles:
//   pos, vel        float4[N]   committed state, original particle order
//   keys            u32[N]      cell key of each particle's prediction (id order)
//   key_s, perm     u32[N]      sorted keys and sorted->original ids
//   pred_a, pred_b  float4[N]   predicted positions in cell order (ping-pong)
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
};

struct FusedShape {
    uint32_t N;
    uint32_t numCells;
    int key_bits;
    int iters;
    bool hashed;
    bool xsph;
};

constexpr unsigned kStatsMaxBlocks = 1024;

// Phase launchers of the fused step (each one graph-capturable).
cudaError_t fused_predict_keys(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);
cudaError_t fused_sort(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);
cudaError_t fused_gather_and_tables(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);
cudaError_t fused_solve(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);
cudaError_t fused_commit(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);
// One kernel of the solve loop: iteration `it`, which = 0 (lambda) or 1
// (delta).  fused_solve == all of them in order.
cudaError_t fused_solve_phase(const FusedBufs& b, const FusedShape& sh, int it, int which, cudaStream_t s);
// Sorted buffer holding the solved prediction after fused_solve.
inline float4* fused_final_pred(const FusedBufs& b, const FusedShape& sh) {
    return (sh.iters % 2 == 0) ? b.pred_a : b.pred_b;
}

// Density statistics of the committed state (fresh grid; uses pred_b/pos_s
// as scratch).  Writes 4 doubles to b.stats_out.
cudaError_t fused_density_stats(const FusedBufs& b, const FusedShape& sh, cudaStream_t s);

// lambda (by original id) of the last iteration, for inspection.
cudaError_t fused_scatter_lambda(const FusedBufs& b, const FusedShape& sh, float* lambda_by_id, cudaStream_t s);

}  // namespace pbf
