// device_buffers.h - device buffers of one simulation (GB300 layout).
//
// Keeps the reference's buffer names (sim/device_buffers.cuh:17-31,
// sim/grid_buffers.cuh:8-28) where the meaning carries over, and adds the
// cell-ordered arrays of the fused GB300 step.  Field meanings:
//   d_pos, d_vel        committed state in ORIGINAL particle order (as the
//                       reference's d_pos / d_vel)
//   d_pos_pred          predicted positions in CELL order (sorted slots);
//                       each solver iteration's delta pass updates them
//   d_pred_alt          (x, y, z, lambda) of the current iteration in cell
//                       order: the lambda pass writes it, the delta pass
//                       reads its neighbours from it (takes the role of the
//                       reference's d_delta)
//   d_pos_sorted        step-start positions in cell order
//   d_vel_sorted        velocities in cell order (velocity phase output)
//   d_lambda            lambda in cell order
//   grid: d_cellKeys (id order), d_cellKeys_sorted, d_indices_sorted (sorted
//   slot -> original id), d_cellLowerBound (numCells+1), compact table.
//
// For launchers registered through KernelDispatcher (KernelLaunchFn): the
// names are the reference's but the layout is not.  A launcher written
// against the reference's sim/device_buffers.cuh reads d_pos_pred and
// d_lambda by particle id; here they are indexed by sorted slot s, whose
// particle is d_indices_sorted[s].  d_delta, d_pos_curr and d_pos_next do not
// exist: the Jacobi update reads the iteration's positions from d_pred_alt
// and writes the next ones over d_pos_pred (SolvedPrediction below gives the
// buffer the Post phase reads), and the commit writes d_pos / d_vel in place.
// tests/cpp/plugin_path.cu is a worked example.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "parameters.h"

namespace sim {

struct DeviceBuffers {
    float4* d_pos = nullptr;
    float4* d_vel = nullptr;
    float4* d_pos_pred = nullptr;
    float4* d_pred_alt = nullptr;
    float4* d_pos_sorted = nullptr;
    float4* d_vel_sorted = nullptr;
    float* d_lambda = nullptr;
    float* d_lambda_by_id = nullptr;  // inspection only
    DeviceParams* d_params = nullptr;  // device-resident parameter block
    uint32_t* d_err = nullptr;         // device error word (bounded waits)
    double* d_stats = nullptr;         // 4 results + per-block partials
    uint32_t capacity = 0;
    bool xsphEnabled = false;  // XSPH post-op configured at initialize (sim/simulator.cpp:277-285)
    // Neighbour lists of the GB300 step (cell order, nbrListCap entries per
    // particle; nbrListCap = 0: no lists, every pass walks the stencil).
    uint32_t* d_nbrList = nullptr;
    uint4* d_tilePlans = nullptr;  // the list build's tile plans, read by the passes after it (scratch)
    uint32_t* d_nbrCount = nullptr;
    uint32_t* d_nbrStats = nullptr;  // [0] longest list built, [1] overflowed lists
    uint32_t nbrListCap = 0;
    // Tile shape of the list passes (particles per CTA and staged slots; the
    // results do not depend on it).
    int tileShape = 0;
    // Arithmetic of the delta pass: 0 exact (bit-identical to the reference
    // kernels), 1 fast (within the 1e-5 bars; PBF_MATH_FAST).
    int mathMode = 0;
    // Fork-join resources of the grid build: after the sort, the gather, the
    // lower-bound table and the compact table each read only the sorted keys,
    // so they run on the step's stream and these two side streams at once
    // (joined back before the lists are built).  Null: one after another.
    cudaStream_t forkStreams[2] = {nullptr, nullptr};
    cudaEvent_t forkEvents[3] = {nullptr, nullptr, nullptr};

    bool allocate(uint32_t cap);
    // (Re)allocates the lists for `capacity` particles; entries is rounded up
    // to a multiple of 8.  On failure the lists are left off (returns false).
    bool allocateLists(uint32_t entries);
    void releaseLists();
    void release();
    ~DeviceBuffers() { release(); }
};

struct GridBuffers {
    uint32_t* d_cellKeys = nullptr;
    uint32_t* d_cellKeys_sorted = nullptr;
    uint32_t* d_indices_sorted = nullptr;
    uint32_t* d_cellLowerBound = nullptr;  // numCells + 1
    uint32_t* d_cellStart = nullptr;       // reference dense format, materialised on request
    uint32_t* d_cellEnd = nullptr;
    uint32_t* d_cellUniqueKeys = nullptr;
    uint32_t* d_cellOffsets = nullptr;  // capacity + 1
    uint32_t* d_compactCount = nullptr;
    void* d_sortTemp = nullptr;
    size_t sortTempBytes = 0;
    void* d_compactTemp = nullptr;
    size_t compactTempBytes = 0;
    uint32_t capacity = 0;
    uint32_t numCells = 0;
    int keyBits = 1;
    bool hashed = false;

    bool allocate(uint32_t cap, uint32_t nCells);
    bool ensureRangesMaterialised();
    void release();
    ~GridBuffers() { release(); }
};

// The prediction the last solver iteration wrote (cell order), i.e. the
// input of the Post phase: d_pos_pred for every iteration count.  (The
// argument is kept so that callers need not change with the buffer scheme.)
inline float4* SolvedPrediction(const DeviceBuffers& b, int /*solverIters*/) { return b.d_pos_pred; }

class KernelDispatcher;

// sim/simulation_context.h:8-20
struct SimulationContext {
    DeviceBuffers* bufs = nullptr;
    GridBuffers* grid = nullptr;
    bool useHashedGrid = false;
    KernelDispatcher* dispatcher = nullptr;
};

}  // namespace sim
