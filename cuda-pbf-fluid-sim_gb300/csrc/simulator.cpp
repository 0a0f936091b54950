// simulator.cpp - sim::Simulator, the phase pipeline and the live dispatcher.
#include "../../include/pbf/simulator.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "fused.cuh"
#include "grid.cuh"
#include "sort.cuh"

namespace sim {

namespace {

template <class T>
bool dalloc(T** p, size_t count) {
    if (count == 0) count = 1;
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * count) == cudaSuccess;
}

template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

int3 compute_dims(const GridBounds& g) {
    const float cs = (g.cellSize > 0.f) ? g.cellSize : 1.f;
    int3 d;
    d.x = int(ceilf((g.maxs.x - g.mins.x) / cs));
    d.y = int(ceilf((g.maxs.y - g.mins.y) / cs));
    d.z = int(ceilf((g.maxs.z - g.mins.z) / cs));
    if (d.x < 0) d.x = 0;
    if (d.y < 0) d.y = 0;
    if (d.z < 0) d.z = 0;
    return d;
}

uint32_t num_cells(int3 d) { return uint32_t(d.x) * uint32_t(d.y) * uint32_t(d.z); }

pbf::FusedBufs fused_bufs(DeviceBuffers& b, GridBuffers& g) {
    pbf::FusedBufs f{};
    f.pos = b.d_pos;
    f.vel = b.d_vel;
    f.keys = g.d_cellKeys;
    f.key_s = g.d_cellKeys_sorted;
    f.perm = g.d_indices_sorted;
    f.pred_a = b.d_pos_pred;
    f.pred_b = b.d_pred_alt;
    f.pos_s = b.d_pos_sorted;
    f.vel_s = b.d_vel_sorted;
    f.lam_s = b.d_lambda;
    f.lb = g.d_cellLowerBound;
    f.uk = g.d_cellUniqueKeys;
    f.off = g.d_cellOffsets;
    f.count = g.d_compactCount;
    f.sort_temp = g.d_sortTemp;
    f.sort_bytes = g.sortTempBytes;
    f.compact_temp = g.d_compactTemp;
    f.compact_bytes = g.compactTempBytes;
    f.dp = b.d_params;
    f.err = b.d_err;
    f.stats_out = b.d_stats;
    f.stats_partials = b.d_stats + 4;
    f.nbr_list = b.d_nbrList;
    f.tile_plans = b.d_tilePlans;
    for (int k = 0; k < 2; ++k) f.fork_streams[k] = b.forkStreams[k];
    for (int k = 0; k < 3; ++k) f.fork_events[k] = b.forkEvents[k];
    f.nbr_count = b.d_nbrCount;
    f.nbr_stats = b.d_nbrStats;
    f.nbr_cap = b.nbrListCap;
    return f;
}

pbf::FusedShape fused_shape(const DeviceBuffers& b, const GridBuffers& g, const SimParams& p) {
    pbf::FusedShape s{};
    s.N = p.numParticles;
    s.numCells = g.numCells;
    s.key_bits = g.keyBits;
    s.iters = p.solverIters;
    s.hashed = g.hashed;
    s.xsph = b.xsphEnabled;
    s.list_span = pbf::list_span_for(p);
    s.tile = b.tileShape;
    s.fast = b.mathMode == 1;
    return s;
}

// ---- built-in GB300 launchers (KernelLaunchFn) ---------------------------
void LaunchIntegrateGB300(DeviceBuffers& b, GridBuffers& g, const SimParams& p, cudaStream_t s) {
    pbf::fused_predict_keys(fused_bufs(b, g), fused_shape(b, g, p), s);
}
void LaunchSortPairsGB300(DeviceBuffers& b, GridBuffers& g, const SimParams& p, cudaStream_t s) {
    pbf::fused_sort(fused_bufs(b, g), fused_shape(b, g, p), s);
}
void LaunchCellRangesGB300(DeviceBuffers& b, GridBuffers& g, const SimParams& p, cudaStream_t s) {
    pbf::fused_gather_and_tables(fused_bufs(b, g), fused_shape(b, g, p), s);
}
void LaunchGridBuildGB300(DeviceBuffers& b, GridBuffers& g, const SimParams& p, cudaStream_t s) {
    LaunchSortPairsGB300(b, g, p, s);
    LaunchCellRangesGB300(b, g, p, s);
}
void LaunchSolveGB300(DeviceBuffers& b, GridBuffers& g, const SimParams& p, cudaStream_t s) {
    pbf::fused_solve(fused_bufs(b, g), fused_shape(b, g, p), s);
}
// The velocity phase is computed by the last solver iteration (or by the
// no-iteration finaliser) in the fused layout.
void LaunchVelocityGB300(DeviceBuffers&, GridBuffers&, const SimParams&, cudaStream_t) {}
void LaunchPostGB300(DeviceBuffers& b, GridBuffers& g, const SimParams& p, cudaStream_t s) {
    pbf::fused_commit(fused_bufs(b, g), fused_shape(b, g, p), s);
}

// ---- phases (sim/phases.cpp:30-106, sim/post_ops.cpp) -------------------
class DispatchedPhase : public IPhase {
public:
    explicit DispatchedPhase(PhaseType t) : m_t(t) {}
    PhaseType type() const override { return m_t; }
    void run(SimulationContext& ctx, const SimParams& p, cudaStream_t s) override {
        if (!ctx.dispatcher) return;
        KernelVariant v;
        v.compact = ctx.useHashedGrid;
        if (KernelLaunchFn fn = ctx.dispatcher->find(v, m_t)) fn(*ctx.bufs, *ctx.grid, p, s);
    }

private:
    PhaseType m_t;
};

}  // namespace

// ------------------------------------------------------------ buffers
bool DeviceBuffers::allocate(uint32_t cap) {
    if (cap == 0) cap = 1;
    if (cap == capacity && d_pos) return true;
    release();
    capacity = cap;
    bool ok = dalloc(&d_pos, cap) && dalloc(&d_vel, cap) && dalloc(&d_pos_pred, cap) && dalloc(&d_pred_alt, cap) &&
              dalloc(&d_pos_sorted, cap) && dalloc(&d_vel_sorted, cap) && dalloc(&d_lambda, cap) &&
              dalloc(&d_lambda_by_id, cap) && dalloc(&d_params, 1) && dalloc(&d_err, 1) &&
              dalloc(&d_stats, 4 + 4 * size_t(pbf::kStatsMaxBlocks));
    if (!ok) {
        release();
        return false;
    }
    cudaMemset(d_pos, 0, sizeof(float4) * cap);
    cudaMemset(d_vel, 0, sizeof(float4) * cap);
    cudaMemset(d_err, 0, sizeof(uint32_t));
    // the clears run on the legacy stream, which the simulator's non-blocking
    // streams do not wait for: finish them before any step is launched
    return cudaDeviceSynchronize() == cudaSuccess;
}

bool DeviceBuffers::allocateLists(uint32_t entries) {
    releaseLists();
    entries = (entries + 7u) & ~7u;
    if (entries == 0 || capacity == 0) return true;
    // whole groups of 32 slots: staged tiles interleave the lists of a group
    const size_t n = size_t((capacity + 31u) & ~31u) * entries;
    if (!dalloc(&d_nbrList, n) || !dalloc(&d_nbrCount, capacity) || !dalloc(&d_nbrStats, 2) ||
        !dalloc(&d_tilePlans, pbf::fused_tile_plan_bytes(capacity) / sizeof(uint4))) {
        releaseLists();
        cudaGetLastError();
        return false;
    }
    cudaMemset(d_nbrStats, 0, 2 * sizeof(uint32_t));
    nbrListCap = entries;
    return cudaDeviceSynchronize() == cudaSuccess;  // as in allocate
}

void DeviceBuffers::releaseLists() {
    dfree(d_nbrList);
    dfree(d_tilePlans);
    dfree(d_nbrCount);
    dfree(d_nbrStats);
    nbrListCap = 0;
}

void DeviceBuffers::release() {
    releaseLists();
    dfree(d_pos);
    dfree(d_vel);
    dfree(d_pos_pred);
    dfree(d_pred_alt);
    dfree(d_pos_sorted);
    dfree(d_vel_sorted);
    dfree(d_lambda);
    dfree(d_lambda_by_id);
    dfree(d_params);
    dfree(d_err);
    dfree(d_stats);
    capacity = 0;
}

bool GridBuffers::allocate(uint32_t cap, uint32_t nCells) {
    release();
    if (cap == 0) cap = 1;
    capacity = cap;
    numCells = nCells;
    keyBits = pbf::bits_for(nCells > 0 ? nCells - 1 : 0);
    sortTempBytes = pbf::sort_temp_bytes(cap, keyBits);
    compactTempBytes = pbf::compact_scratch_bytes(cap);
    bool ok = dalloc(&d_cellKeys, cap) && dalloc(&d_cellKeys_sorted, cap) && dalloc(&d_indices_sorted, cap) &&
              dalloc(&d_cellLowerBound, size_t(nCells) + 1) && dalloc(&d_cellUniqueKeys, cap) &&
              dalloc(&d_cellOffsets, size_t(cap) + 1) && dalloc(&d_compactCount, 1) &&
              cudaMalloc(&d_sortTemp, sortTempBytes) == cudaSuccess &&
              cudaMalloc(&d_compactTemp, compactTempBytes) == cudaSuccess;
    if (!ok) {
        release();
        return false;
    }
    cudaMemset(d_compactCount, 0, sizeof(uint32_t));
    return cudaDeviceSynchronize() == cudaSuccess;  // as in DeviceBuffers::allocate
}

bool GridBuffers::ensureRangesMaterialised() {
    if (d_cellStart && d_cellEnd) return true;
    return dalloc(&d_cellStart, numCells) && dalloc(&d_cellEnd, numCells);
}

void GridBuffers::release() {
    dfree(d_cellKeys);
    dfree(d_cellKeys_sorted);
    dfree(d_indices_sorted);
    dfree(d_cellLowerBound);
    dfree(d_cellStart);
    dfree(d_cellEnd);
    dfree(d_cellUniqueKeys);
    dfree(d_cellOffsets);
    dfree(d_compactCount);
    if (d_sortTemp) cudaFree(d_sortTemp);
    if (d_compactTemp) cudaFree(d_compactTemp);
    d_sortTemp = d_compactTemp = nullptr;
    sortTempBytes = compactTempBytes = 0;
    capacity = 0;
}

// ---------------------------------------------------------- dispatcher
void InitializeKernelDispatcher(KernelDispatcher& kd) {
    for (bool compact : {false, true}) {
        kd.registerKernel(PhaseType::Integrate, false, false, compact, LaunchIntegrateGB300);
        kd.registerKernel(PhaseType::GridBuild, false, false, compact, LaunchGridBuildGB300);
        kd.registerKernel(PhaseType::SortPairs, false, false, compact, LaunchSortPairsGB300);
        kd.registerKernel(PhaseType::CellRanges, false, false, compact, LaunchCellRangesGB300);
        kd.registerKernel(PhaseType::SolveIterations, false, false, compact, LaunchSolveGB300);
        kd.registerKernel(PhaseType::Velocity, false, false, compact, LaunchVelocityGB300);
        kd.registerKernel(PhaseType::Post, false, false, compact, LaunchPostGB300);
    }
}

void BuildDefaultPipelines(PhasePipeline& pipeline) {
    pipeline.clear();
    pipeline.addFull(std::make_unique<DispatchedPhase>(PhaseType::Integrate));
    pipeline.addFull(std::make_unique<DispatchedPhase>(PhaseType::GridBuild));
    pipeline.addFull(std::make_unique<DispatchedPhase>(PhaseType::SolveIterations));
    pipeline.addFull(std::make_unique<DispatchedPhase>(PhaseType::Velocity));
    pipeline.addFull(std::make_unique<DispatchedPhase>(PhaseType::Post));
}

// ------------------------------------------------------ change tracker
void ParamChangeTracker::capture(const SimParams& p, uint32_t numCells) {
    m_numParticles = p.numParticles;
    m_solverIters = p.solverIters;
    m_maxNeighbors = p.maxNeighbors;
    m_numCells = numCells;
    m_grid = p.grid;
    m_xsph = p.xsph_c > 0.f;
    m_listSpan = pbf::list_span_for(p);
}

bool ParamChangeTracker::structuralChanged(const SimParams& p, uint32_t numCells) const {
    if (p.solverIters != m_solverIters) return true;
    if (p.maxNeighbors != m_maxNeighbors) return true;
    if (p.numParticles != m_numParticles) return true;
    if (numCells != m_numCells) return true;
    if (p.grid.dim.x != m_grid.dim.x || p.grid.dim.y != m_grid.dim.y || p.grid.dim.z != m_grid.dim.z) return true;
    if (pbf::list_span_for(p) != m_listSpan) return true;  // list builds are part of the graph
    return false;
}

// ----------------------------------------------------------- simulator
Simulator::Simulator() = default;
Simulator::~Simulator() { shutdown(); }

bool Simulator::initialize(const SimParams& p, bool useHashedGrid) {
    shutdown();
    m_params = p;
    m_params.grid.dim = compute_dims(p.grid);
    m_useHashedGrid = useHashedGrid;
    const uint32_t nc = num_cells(m_params.grid.dim);
    if (nc == 0) return false;
    if (cudaStreamCreateWithFlags(&m_ownStream, cudaStreamNonBlocking) != cudaSuccess) return false;
    m_stream = m_ownStream;
    for (cudaStream_t& fs : m_bufs.forkStreams)
        if (cudaStreamCreateWithFlags(&fs, cudaStreamNonBlocking) != cudaSuccess) return false;
    for (cudaEvent_t& fe : m_bufs.forkEvents)
        if (cudaEventCreateWithFlags(&fe, cudaEventDisableTiming) != cudaSuccess) return false;
    uint32_t cap = std::max(p.maxParticles, p.numParticles);
    if (cap == 0) cap = 1;
    if (!m_bufs.allocate(cap)) return false;
    if (!m_grid.allocate(cap, nc)) return false;
    m_bufs.allocateLists(m_listCapacity);  // lists stay off if this fails
    if (pbf::fused_prepare_kernels() != cudaSuccess) return false;
    m_grid.hashed = useHashedGrid;
    m_bufs.xsphEnabled = (p.xsph_c > 0.f);
    m_kernelDispatcher = KernelDispatcher{};
    InitializeKernelDispatcher(m_kernelDispatcher);
    BuildDefaultPipelines(m_pipeline);
    m_ctx.bufs = &m_bufs;
    m_ctx.grid = &m_grid;
    m_ctx.useHashedGrid = useHashedGrid;
    m_ctx.dispatcher = &m_kernelDispatcher;
    m_paramsValid = false;
    m_graphDirty = true;
    if (!uploadParamsIfChanged()) return false;
    m_paramTracker.capture(m_params, nc);
    return cudaDeviceSynchronize() == cudaSuccess;
}

void Simulator::shutdown() {
    destroyGraph();
    if (m_stream) cudaStreamSynchronize(m_stream);
    if (m_ownStream) {
        cudaStreamSynchronize(m_ownStream);
        cudaStreamDestroy(m_ownStream);
        m_ownStream = nullptr;
    }
    m_stream = nullptr;
    for (cudaStream_t& fs : m_bufs.forkStreams)
        if (fs) {
            cudaStreamSynchronize(fs);
            cudaStreamDestroy(fs);
            fs = nullptr;
        }
    for (cudaEvent_t& fe : m_bufs.forkEvents)
        if (fe) {
            cudaEventDestroy(fe);
            fe = nullptr;
        }
    m_bufs.release();
    m_grid.release();
    m_paramsValid = false;
}

void Simulator::destroyGraph() {
    if (m_graphExec) cudaGraphExecDestroy(m_graphExec);
    if (m_graph) cudaGraphDestroy(m_graph);
    m_graphExec = nullptr;
    m_graph = nullptr;
}

bool Simulator::uploadParamsIfChanged() {
    DeviceParams dp = MakeDeviceParams(m_params);
    if (m_paramsValid && std::memcmp(&dp, &m_uploaded, sizeof(dp)) == 0) return true;
    // Pageable source: the runtime stages it before returning, so the host
    // struct may change right after; ordered before the next graph launch.
    if (cudaMemcpyAsync(m_bufs.d_params, &dp, sizeof(dp), cudaMemcpyHostToDevice, m_stream) != cudaSuccess)
        return false;
    m_uploaded = dp;
    m_paramsValid = true;
    return true;
}

bool Simulator::ensureCapacity(uint32_t n) {
    if (n <= m_bufs.capacity) return true;
    cudaStreamSynchronize(m_stream);
    // Keep the committed state across the reallocation.
    std::vector<float4> pos(m_bufs.capacity), vel(m_bufs.capacity);
    cudaMemcpy(pos.data(), m_bufs.d_pos, sizeof(float4) * pos.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(vel.data(), m_bufs.d_vel, sizeof(float4) * vel.size(), cudaMemcpyDeviceToHost);
    const bool xs = m_bufs.xsphEnabled;
    if (!m_bufs.allocate(n) || !m_grid.allocate(n, m_grid.numCells)) return false;
    m_bufs.allocateLists(m_listCapacity);
    m_bufs.xsphEnabled = xs;
    m_grid.hashed = m_useHashedGrid;
    // on the simulator's stream (non-blocking: the legacy stream's copies are
    // not ordered before its launches); a pageable source is staged before
    // the call returns
    cudaMemcpyAsync(m_bufs.d_pos, pos.data(), sizeof(float4) * pos.size(), cudaMemcpyHostToDevice, m_stream);
    cudaMemcpyAsync(m_bufs.d_vel, vel.data(), sizeof(float4) * vel.size(), cudaMemcpyHostToDevice, m_stream);
    m_paramsValid = false;
    m_graphDirty = true;
    return true;
}

bool Simulator::captureGraph() {
    destroyGraph();
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(m_ownStream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
    m_pipeline.runFull(m_ctx, m_params, m_ownStream);
    cudaError_t e = cudaStreamEndCapture(m_ownStream, &g);
    if (e != cudaSuccess || !g) {
        cudaGetLastError();
        return false;
    }
    if (cudaGraphInstantiate(&m_graphExec, g, 0) != cudaSuccess) {
        cudaGraphDestroy(g);
        m_graphExec = nullptr;
        return false;
    }
    m_graph = g;
    cudaGraphUpload(m_graphExec, m_stream);
    m_graphDirty = false;
    return true;
}

bool Simulator::step(const SimParams& p) {
    if (!m_stream) return false;
    SimParams np = p;
    np.grid.dim = compute_dims(p.grid);
    const uint32_t nc = num_cells(np.grid.dim);
    if (nc == 0) return false;
    if (!ensureCapacity(np.numParticles)) return false;
    if (nc != m_grid.numCells) {
        cudaStreamSynchronize(m_stream);
        const uint32_t cap = m_grid.capacity;
        if (!m_grid.allocate(cap, nc)) return false;
        m_grid.hashed = m_useHashedGrid;
        m_graphDirty = true;
    }
    if (m_paramTracker.structuralChanged(np, nc)) m_graphDirty = true;
    m_params = np;
    if (!uploadParamsIfChanged()) return false;
    if (m_graphDirty) {
        if (!captureGraph()) return false;
        m_paramTracker.capture(m_params, nc);
    }
    if (cudaGraphLaunch(m_graphExec, m_stream) != cudaSuccess) return false;
    ++m_frameIndex;
    return true;
}

bool Simulator::setStream(cudaStream_t s) {
    if (!m_ownStream) return false;
    const cudaStream_t next = s ? s : m_ownStream;
    if (next == m_stream) return true;
    if (cudaStreamSynchronize(m_stream) != cudaSuccess) return false;
    m_stream = next;
    return true;
}

int Simulator::launchesPerStep() const {
    const int passes = (m_grid.keyBits + 7) / 8;
    int n = 1 /*predict_keys*/ + 1 /*hist*/ + passes + 1 /*gather*/ + (m_params.numParticles > 0 ? 2 : 1) /*lb mark, fill*/;
    if (m_grid.hashed) n += 1;
    n += (m_params.solverIters > 0) ? 2 * m_params.solverIters : 1;
    if (m_bufs.nbrListCap > 0) n += pbf::fused_list_builds(fused_shape(m_bufs, m_grid, m_params));
    n += 1; /*commit*/
    return n;
}

bool Simulator::setMathMode(int mode) {
    if (mode != 0 && mode != 1) return false;
    if (mode == m_bufs.mathMode) return true;
    if (m_stream) cudaStreamSynchronize(m_stream);
    m_bufs.mathMode = mode;
    m_graphDirty = true;
    return true;
}

bool Simulator::setTileShape(int id) {
    if (id < 0 || id >= pbf::fused_tile_shape_count()) return false;
    if (id == m_bufs.tileShape) return true;
    if (m_stream) cudaStreamSynchronize(m_stream);
    m_bufs.tileShape = id;
    m_graphDirty = true;
    return true;
}

bool Simulator::autotuneTileShape(const SimParams& p, int steps, float* ms) {
    if (!m_stream || steps < 1 || p.numParticles > m_bufs.capacity) return false;
    const uint32_t n = p.numParticles;
    const int shapes = pbf::fused_tile_shape_count();
    const int before = m_bufs.tileShape;
    const uint64_t frame = m_frameIndex;
    // every shape starts from the state as it is now, and the call leaves it so
    float4* snap = nullptr;
    const size_t bytes = sizeof(float4) * size_t(n);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool ok = cudaStreamSynchronize(m_stream) == cudaSuccess &&
              cudaMalloc(&snap, 2 * std::max<size_t>(bytes, 16)) == cudaSuccess &&
              cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(snap, m_bufs.d_pos, bytes, cudaMemcpyDeviceToDevice, m_stream) == cudaSuccess &&
         cudaMemcpyAsync(snap + n, m_bufs.d_vel, bytes, cudaMemcpyDeviceToDevice, m_stream) == cudaSuccess;
    auto restore = [&]() {
        return cudaMemcpyAsync(m_bufs.d_pos, snap, bytes, cudaMemcpyDeviceToDevice, m_stream) == cudaSuccess &&
               cudaMemcpyAsync(m_bufs.d_vel, snap + n, bytes, cudaMemcpyDeviceToDevice, m_stream) == cudaSuccess;
    };
    std::vector<float> times(size_t(shapes), 0.f);
    for (int id = 0; ok && id < shapes; ++id) {
        // one untimed step captures the shape's graph
        ok = setTileShape(id) && step(p) && restore() && cudaEventRecord(e0, m_stream) == cudaSuccess;
        for (int i = 0; ok && i < steps; ++i) ok = step(p);
        float t = 0.f;
        ok = ok && cudaEventRecord(e1, m_stream) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
             cudaEventElapsedTime(&t, e0, e1) == cudaSuccess && restore();
        if (!ok) break;
        times[size_t(id)] = t / float(steps);
        if (ms) ms[id] = times[size_t(id)];
    }
    const int best = ok ? pbf::pick_tile_shape(times.data(), shapes, before) : before;
    if (snap) ok = restore() && cudaStreamSynchronize(m_stream) == cudaSuccess && ok;
    m_frameIndex = frame;
    setTileShape(best);
    uint32_t l = 0, o = 0;
    neighbourListStats(l, o, true);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (snap) cudaFree(snap);
    return ok;
}

bool Simulator::setNeighbourListCapacity(uint32_t entries) {
    if (m_stream) cudaStreamSynchronize(m_stream);
    m_listCapacity = (entries + 7u) & ~7u;
    m_graphDirty = true;
    if (m_bufs.capacity == 0) return true;
    return m_bufs.allocateLists(m_listCapacity);
}

bool Simulator::neighbourListStats(uint32_t& longest, uint32_t& overflowed, bool reset) {
    longest = overflowed = 0;
    if (!m_bufs.d_nbrStats) return m_bufs.nbrListCap == 0;
    if (m_stream) cudaStreamSynchronize(m_stream);
    uint32_t v[2] = {0, 0};
    if (cudaMemcpy(v, m_bufs.d_nbrStats, sizeof(v), cudaMemcpyDeviceToHost) != cudaSuccess) return false;
    longest = v[0];
    overflowed = v[1];
    if (reset) cudaMemsetAsync(m_bufs.d_nbrStats, 0, sizeof(v), m_stream);
    return true;
}

int Simulator::profileStep(const SimParams& p, float* ms, const char** names, int cap) {
    // Bring buffers/params up to date exactly like step(), then capture the
    // phases with external event-record nodes between them into one graph:
    // the events time the device work only (no host enqueue gaps).
    SimParams np = p;
    np.grid.dim = compute_dims(p.grid);
    const uint32_t nc = num_cells(np.grid.dim);
    if (nc == 0 || nc != m_grid.numCells || !ensureCapacity(np.numParticles)) return -1;
    m_params = np;
    if (!uploadParamsIfChanged()) return -1;
    pbf::FusedBufs b = fused_bufs(m_bufs, m_grid);
    pbf::FusedShape sh = fused_shape(m_bufs, m_grid, m_params);
    static const char* kIterNames[3][8] = {
        {"lambda_1", "lambda_2", "lambda_3", "lambda_4", "lambda_5", "lambda_6", "lambda_7", "lambda_8"},
        {"delta_1", "delta_2", "delta_3", "delta_4", "delta_5", "delta_6", "delta_7", "delta_8"},
        {"lists_1", "lists_2", "lists_3", "lists_4", "lists_5", "lists_6", "lists_7", "lists_8"}};
    // captured on the owned stream, launched on the current one
    const cudaStream_t cs = m_ownStream;
    std::vector<cudaEvent_t> ev;
    std::vector<const char*> nm;
    auto mark = [&](const char* name) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecordWithFlags(e, cs, cudaEventRecordExternal);
        ev.push_back(e);
        if (name) nm.push_back(name);
    };
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return -1;
    mark(nullptr);
    pbf::fused_predict_keys(b, sh, cs);
    mark("predict_keys");
    pbf::fused_sort(b, sh, cs);
    mark("sort");
    pbf::fused_gather_and_tables(b, sh, cs);
    mark("gather_tables");
    if (sh.iters > 8) {
        pbf::fused_solve(b, sh, cs);
        mark("solve");
    } else if (sh.iters <= 0) {
        pbf::fused_solve(b, sh, cs);
        mark("finalize");
    } else {
        for (int it = 0; it < sh.iters; ++it) {
            if (pbf::fused_build_lists(b, sh, it, cs) == cudaSuccess) mark(kIterNames[2][it]);
            pbf::fused_solve_phase(b, sh, it, 0, cs);
            mark(kIterNames[0][it]);
            pbf::fused_solve_phase(b, sh, it, 1, cs);
            mark(kIterNames[1][it]);
        }
    }
    pbf::fused_commit(b, sh, cs);
    mark("commit");
    int n = 0;
    cudaGraphExec_t exec = nullptr;
    if (cudaStreamEndCapture(cs, &graph) == cudaSuccess && graph &&
        cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess && cudaGraphLaunch(exec, m_stream) == cudaSuccess &&
        cudaStreamSynchronize(m_stream) == cudaSuccess) {
        for (size_t k = 1; k < ev.size() && n < cap; ++k, ++n) {
            if (cudaEventElapsedTime(&ms[n], ev[k - 1], ev[k]) != cudaSuccess) ms[n] = -1.f;
            if (names) names[n] = nm[k - 1];
        }
    } else {
        n = -1;
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    cudaGetLastError();
    return n;
}

uint32_t Simulator::takeDeviceError() {
    if (!m_bufs.d_err) return 0;
    uint32_t e = 0;
    cudaStreamSynchronize(m_stream);
    cudaMemcpy(&e, m_bufs.d_err, sizeof(e), cudaMemcpyDeviceToHost);
    // cleared on the simulator's stream, so the clear is ordered before the
    // next step's launches (which run on that stream, not the legacy one)
    if (e) cudaMemsetAsync(m_bufs.d_err, 0, sizeof(uint32_t), m_stream);
    return e;
}

void Simulator::syncForRender() {
    if (m_stream) cudaStreamSynchronize(m_stream);
}

void Simulator::uploadPositions(const std::vector<float4>& pos, const std::vector<float4>* vel) {
    const uint32_t n = uint32_t(pos.size());
    ensureCapacity(n);
    cudaStreamSynchronize(m_stream);
    // ordered on the simulator's stream before the next step (see ensureCapacity)
    cudaMemcpyAsync(m_bufs.d_pos, pos.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, m_stream);
    if (vel)
        cudaMemcpyAsync(m_bufs.d_vel, vel->data(), sizeof(float4) * n, cudaMemcpyHostToDevice, m_stream);
    else
        cudaMemsetAsync(m_bufs.d_vel, 0, sizeof(float4) * n, m_stream);
    cudaStreamSynchronize(m_stream);  // blocking, as the reference's upload
    if (m_params.numParticles != n) m_graphDirty = true;
    m_params.numParticles = n;
}

// sim/simulator.cpp:808-877 (lattice, clamped into the box, w = 1).
void Simulator::seedBoxLattice(uint32_t nx, uint32_t ny, uint32_t nz, float3 origin, float spacing) {
    const uint64_t n64 = uint64_t(nx) * ny * nz;
    const uint32_t N = n64 > 0xFFFFFFFFull ? 0xFFFFFFFFu : uint32_t(n64);
    std::vector<float4> pos(N);
    const GridBounds& g = m_params.grid;
    uint32_t idx = 0;
    for (uint32_t iz = 0; iz < nz && idx < N; ++iz)
        for (uint32_t iy = 0; iy < ny && idx < N; ++iy)
            for (uint32_t ix = 0; ix < nx && idx < N; ++ix) {
                float x = origin.x + float(ix) * spacing;
                float y = origin.y + float(iy) * spacing;
                float z = origin.z + float(iz) * spacing;
                x = fminf(fmaxf(x, g.mins.x), g.maxs.x);
                y = fminf(fmaxf(y, g.mins.y), g.maxs.y);
                z = fminf(fmaxf(z, g.mins.z), g.maxs.z);
                pos[idx++] = make_float4(x, y, z, 1.0f);
            }
    uploadPositions(pos, nullptr);
}

// sim/simulator.cpp:880-934 (lattice dims fitted to the domain).
void Simulator::seedBoxLatticeAuto(uint32_t total, float3 origin, float spacing) {
    const GridBounds& g = m_params.grid;
    const float sx = fmaxf(0.f, g.maxs.x - g.mins.x), sy = fmaxf(0.f, g.maxs.y - g.mins.y),
                sz = fmaxf(0.f, g.maxs.z - g.mins.z);
    auto cap = [&](float len) -> uint32_t { return (spacing > 0.f) ? uint32_t(floorf(len / spacing)) : 0u; };
    const uint32_t maxX = std::max<uint32_t>(1, cap(sx)), maxY = std::max<uint32_t>(1, cap(sy)),
                   maxZ = std::max<uint32_t>(1, cap(sz));
    const uint64_t T = std::max<uint32_t>(1u, total);
    uint32_t nx = std::min<uint32_t>(maxX, uint32_t(std::ceil(std::pow(double(T), 1.0 / 3.0))));
    const uint64_t remXY = (T + nx - 1) / nx;
    uint32_t ny = std::min<uint32_t>(maxY, uint32_t(std::ceil(std::sqrt(double(remXY)))));
    uint32_t nz = std::min<uint32_t>(maxZ, uint32_t(std::ceil(double(remXY) / std::max<uint32_t>(1u, ny))));
    while (uint64_t(nx) * ny * nz < T) {
        if (nx < maxX) ++nx;
        else if (ny < maxY) ++ny;
        else if (nz < maxZ) ++nz;
        else break;
    }
    const float m = spacing * 0.25f;
    origin.x = fminf(fmaxf(origin.x, g.mins.x + m), g.maxs.x - m);
    origin.y = fminf(fmaxf(origin.y, g.mins.y + m), g.maxs.y - m);
    origin.z = fminf(fmaxf(origin.z, g.mins.z + m), g.maxs.z - m);
    seedBoxLattice(nx, ny, nz, origin, spacing);
}

// sim/simulator.cpp:963-1040 (cube groups, w = group index, optional
// unit-sphere rejection jitter from std::mt19937(jitterSeed)).
void Simulator::seedCubeMix(uint32_t groupCount, const float3* centers, uint32_t edge, float spacing,
                            bool applyJitter, float jitterAmp, uint32_t jitterSeed) {
    if (groupCount == 0 || edge == 0) {
        uploadPositions({}, nullptr);
        return;
    }
    const uint64_t per = uint64_t(edge) * edge * edge;
    const uint64_t t64 = per * groupCount;
    const uint32_t total = t64 > 0xFFFFFFFFull ? 0xFFFFFFFFu : uint32_t(t64);
    std::vector<float4> pos(total);
    const GridBounds& g = m_params.grid;
    uint32_t cur = 0;
    for (uint32_t gi = 0; gi < groupCount && cur < total; ++gi) {
        const float3 c = centers[gi];
        const float start = -0.5f * spacing * float(edge - 1);
        for (uint32_t iz = 0; iz < edge && cur < total; ++iz)
            for (uint32_t iy = 0; iy < edge && cur < total; ++iy)
                for (uint32_t ix = 0; ix < edge && cur < total; ++ix) {
                    float x = c.x + start + float(ix) * spacing;
                    float y = c.y + start + float(iy) * spacing;
                    float z = c.z + start + float(iz) * spacing;
                    x = fminf(fmaxf(x, g.mins.x), g.maxs.x);
                    y = fminf(fmaxf(y, g.mins.y), g.maxs.y);
                    z = fminf(fmaxf(z, g.mins.z), g.maxs.z);
                    pos[cur++] = make_float4(x, y, z, float(gi));
                }
    }
    if (applyJitter && jitterAmp > 0.f) {
        std::mt19937 rng(jitterSeed);
        std::uniform_real_distribution<float> U(-1.f, 1.f);
        for (uint32_t i = 0; i < total; ++i) {
            float ox, oy, oz;
            for (;;) {
                ox = U(rng);
                oy = U(rng);
                oz = U(rng);
                if (ox * ox + oy * oy + oz * oz <= 1.f) break;
            }
            float4 p = pos[i];
            p.x = fminf(fmaxf(p.x + ox * jitterAmp, g.mins.x), g.maxs.x);
            p.y = fminf(fmaxf(p.y + oy * jitterAmp, g.mins.y), g.maxs.y);
            p.z = fminf(fmaxf(p.z + oz * jitterAmp, g.mins.z), g.maxs.z);
            pos[i] = p;
        }
    }
    uploadPositions(pos, nullptr);
}

bool Simulator::computeCenterOfMass(float3& out, uint32_t stride) const {
    out = make_float3(0, 0, 0);
    const uint32_t N = m_params.numParticles;
    if (N == 0) return true;
    std::vector<float4> h(N);
    cudaStreamSynchronize(m_stream);
    if (cudaMemcpy(h.data(), m_bufs.d_pos, sizeof(float4) * N, cudaMemcpyDeviceToHost) != cudaSuccess) return false;
    const uint32_t st = stride == 0 ? 1u : stride;
    double sx = 0, sy = 0, sz = 0;
    uint64_t cnt = 0;
    for (uint32_t i = 0; i < N; i += st) {
        sx += h[i].x;
        sy += h[i].y;
        sz += h[i].z;
        ++cnt;
    }
    out = make_float3(float(sx / cnt), float(sy / cnt), float(sz / cnt));
    return true;
}

}  // namespace sim
