// simulator.h - sim::Simulator, the headless GB300 step pipeline.
//
// Keeps the reference's public surface (sim/simulator.h:47-91) minus the
// D3D12 interop members: initialize / step / shutdown, seeding helpers and
// buffer accessors.  step() launches one CUDA graph holding the whole step
// (the reference captures the same phase sequence, sim/graph_builder.cpp:
// 60-62) and commits the new state in place, so no ping-pong swap is needed.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "device_buffers.h"
#include "kernel_dispatcher.h"
#include "parameters.h"

namespace sim {

// sim/phase_pipeline.h:14-19
class IPhase {
public:
    virtual ~IPhase() = default;
    virtual PhaseType type() const = 0;
    virtual void run(SimulationContext& ctx, const SimParams& params, cudaStream_t stream) = 0;
};

// sim/phase_pipeline.h:21-39: full = integrate, grid build, solve, velocity,
// then the post stage (XSPH -> boundary -> commit, sim/post_ops.cpp:73-85).
class PhasePipeline {
public:
    void addFull(std::unique_ptr<IPhase> p) { m_full.push_back(std::move(p)); }
    const std::vector<std::unique_ptr<IPhase>>& full() const { return m_full; }
    void runFull(SimulationContext& ctx, const SimParams& p, cudaStream_t s) {
        for (auto& ph : m_full) ph->run(ctx, p, s);
    }
    void clear() { m_full.clear(); }

private:
    std::vector<std::unique_ptr<IPhase>> m_full;
};

// Populates the default phase list (sim/phases.cpp:108-117 order).
void BuildDefaultPipelines(PhasePipeline& pipeline);

// Structural vs dynamic parameter changes (sim/param_change_tracker.h:8-56).
// Structural changes re-capture the step graph; every other change is
// written to the device-resident parameter block before the next launch.
class ParamChangeTracker {
public:
    void capture(const SimParams& p, uint32_t numCells);
    bool structuralChanged(const SimParams& p, uint32_t numCells) const;

private:
    uint32_t m_numParticles = 0;
    int m_solverIters = -1;
    int m_maxNeighbors = 0;
    uint32_t m_numCells = 0;
    GridBounds m_grid{};
    bool m_xsph = false;
    int m_listSpan = -1;
};

class Simulator {
public:
    Simulator();
    ~Simulator();
    Simulator(const Simulator&) = delete;
    Simulator& operator=(const Simulator&) = delete;

    // sim/simulator.cpp:217-296.  useHashedGrid selects the compact table
    // (the reference reads it from console perf.use_hashed_grid).
    bool initialize(const SimParams& p, bool useHashedGrid = true);
    void shutdown();
    // One step on the simulator's stream (asynchronous).
    bool step(const SimParams& p);

    // Runs the simulator's work on a caller's stream from now on (nullptr:
    // back to the stream the simulator owns).  The switch waits for the work
    // already queued on the old stream.  Graphs are still captured on the
    // owned stream and launched on the current one.
    bool setStream(cudaStream_t s);

    // Accessors (original particle order).
    const float4* devicePositions() const { return m_bufs.d_pos; }
    float4* renderPositionPtr() const { return m_bufs.d_pos; }
    const float4* deviceVel() const { return m_bufs.d_vel; }
    float4* devicePositionsMutable() { return m_bufs.d_pos; }
    float4* deviceVelMutable() { return m_bufs.d_vel; }
    uint32_t activeParticleCount() const { return m_params.numParticles; }
    const SimParams& params() const { return m_params; }
    cudaStream_t cudaStream() const { return m_stream; }
    uint32_t numCells() const { return m_grid.numCells; }
    bool hashedGrid() const { return m_useHashedGrid; }
    DeviceBuffers& buffers() { return m_bufs; }
    GridBuffers& gridBuffers() { return m_grid; }
    KernelDispatcher& dispatcher() { return m_kernelDispatcher; }
    PhasePipeline& pipeline() { return m_pipeline; }

    // Seeding (sim/simulator.cpp:808-1040).  Host generation + upload; the
    // lattice is clamped into the grid box, w = 1, velocities zeroed.
    void seedBoxLattice(uint32_t nx, uint32_t ny, uint32_t nz, float3 origin, float spacing);
    void seedBoxLatticeAuto(uint32_t total, float3 origin, float spacing);
    void seedCubeMix(uint32_t groupCount, const float3* groupCenters, uint32_t edgeParticles, float spacing,
                     bool applyJitter, float jitterAmp, uint32_t jitterSeed);
    bool computeCenterOfMass(float3& outCom, uint32_t sampleStride) const;
    void syncForRender();

    // Forces the step graph to be re-captured at the next step (e.g. after a
    // launcher was registered in the dispatcher).
    void invalidateGraph() { m_graphDirty = true; }
    // Device error word: returns and clears it (0 = no error).
    uint32_t takeDeviceError();
    // One step launched phase by phase with events in between (profiling);
    // returns the number of phases written to ms/names.
    int profileStep(const SimParams& p, float* ms, const char** names, int cap);
    // Kernel launches of this library per step for the current shape.
    int launchesPerStep() const;

    // Neighbour lists (no counterpart in the reference).  Each solver pass
    // of the GB300 step walks a per-particle list of the stencil candidates
    // near it instead of the whole 27-cell stencil; results are identical.
    // entries = list capacity per particle (rounded up to a multiple of 8;
    // particles with more candidates walk the stencil); 0 turns lists off.
    // Device memory: 4 * entries bytes per particle.
    bool setNeighbourListCapacity(uint32_t entries);
    uint32_t neighbourListCapacity() const { return m_bufs.nbrListCap; }
    // Longest list built and number of overflowed lists since the last reset.
    bool neighbourListStats(uint32_t& longest, uint32_t& overflowed, bool reset);
    static constexpr uint32_t kDefaultListCapacity = 512;

    // Tile shape of the list passes (no counterpart in the reference): how
    // many sorted particles a CTA takes and how many neighbour slots it can
    // stage in shared memory.  Every shape gives the same results; the fastest
    // depends on the scene.  setTileShape takes effect at the next step.
    bool setTileShape(int id);
    int tileShape() const { return m_bufs.tileShape; }
    // Arithmetic of the delta pass: 0 exact (the default; bit-identical to
    // the reference kernels), 1 fast (the s_corr power from error-free
    // products instead of powf; per-step state within 1e-5 relative).  Takes effect at the next
    // step (the step graph is captured again).
    bool setMathMode(int mode);
    int mathMode() const { return m_bufs.mathMode; }
    // Times `steps` steps of every tile shape from the current state (after
    // one untimed step per shape), then puts the state back as it was,
    // clears the list statistics and keeps the fastest shape.  ms (tile
    // shape count entries, may be null) receives each shape's mean step time.
    bool autotuneTileShape(const SimParams& p, int steps, float* ms);

private:
    bool ensureCapacity(uint32_t n);
    bool uploadParamsIfChanged();
    bool captureGraph();
    void destroyGraph();
    void uploadPositions(const std::vector<float4>& pos, const std::vector<float4>* vel);

    SimParams m_params{};
    DeviceParams m_uploaded{};
    bool m_paramsValid = false;
    DeviceBuffers m_bufs{};
    GridBuffers m_grid{};
    bool m_useHashedGrid = true;
    cudaStream_t m_stream = nullptr;     // where work is enqueued (owned or a caller's)
    cudaStream_t m_ownStream = nullptr;  // created by initialize; graphs are captured here
    cudaGraph_t m_graph = nullptr;
    cudaGraphExec_t m_graphExec = nullptr;
    bool m_graphDirty = true;
    ParamChangeTracker m_paramTracker;
    KernelDispatcher m_kernelDispatcher;
    PhasePipeline m_pipeline;
    SimulationContext m_ctx;
    uint64_t m_frameIndex = 0;
    uint32_t m_listCapacity = kDefaultListCapacity;
};

}  // namespace sim
