// ensemble.cu - many independent scenes stepped as one workload.
//
// The reference steps one scene per sim::Simulator (sim/simulator.cpp:560-643);
// a batch of scenes is a loop over simulators, each step a dozen small launches
// that leave most of the GPU idle for scenes of a few thousand particles.  Here
// the scenes' particles are concatenated (scene s owns ids [off[s], off[s+1]))
// and every phase is one launch over all of them:
//   * cell keys are global: scene s's cells are numbered from cellOff[s], so a
//     single stable sort of the keys orders particles by (scene, cell, id), the
//     order each scene's own sort produces, and one lower-bound table over all
//     scenes' cells gives every scene its cell ranges;
//   * each particle reads its scene's parameter block (grid, gravity, dt,
//     kernel, tuning, iteration count); a warp may hold particles of two
//     scenes, which the per-lane walks allow;
//   * the neighbour passes are the simulator's own list kernels with a
//     per-slot scene lookup (fused.cu): lists built once per step for the
//     scenes whose single-list schedule holds, tiles of one scene row staged
//     in shared memory;
//   * scenes with fewer solver iterations than the ensemble's maximum carry
//     their prediction through the remaining passes unchanged.
// Every scene therefore evolves bit-identically to a pbf_sim of the same
// parameters.  The step is one CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/pbf/pbf.h"
#include "../../include/pbf/simulator.h"
#include "fused.cuh"
#include "grid.cuh"
#include "pbf_common.cuh"
#include "sort.cuh"

namespace pbf {
namespace {

constexpr int kBS = 256;
__global__ void __launch_bounds__(kBS) k_ens_predict_keys(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                          const SceneInfo* __restrict__ scenes,
                                                          const uint32_t* __restrict__ sceneOfId, uint32_t N,
                                                          uint32_t* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const SceneInfo& sc = scenes[sceneOfId[i]];
    const float4 x = predict_clamped(pos[i], vel[i], sc.dp.gravity, sc.dp.dt, sc.dp.grid);
    keys[i] = sc.cellOffset + cell_key(x, sc.dp.grid);
}

__global__ void __launch_bounds__(kBS) k_ens_gather(const uint32_t* __restrict__ perm, const float4* __restrict__ pos,
                                                    const float4* __restrict__ vel,
                                                    const SceneInfo* __restrict__ scenes,
                                                    const uint32_t* __restrict__ sceneOfId, uint32_t N,
                                                    float4* __restrict__ pred_s, float4* __restrict__ pos_s,
                                                    uint32_t* __restrict__ sceneOfSlot) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const uint32_t i = perm[s];
    const uint32_t sc = sceneOfId[i];
    const float4 p = pos[i];
    pred_s[s] = predict_clamped(p, vel[i], scenes[sc].dp.gravity, scenes[sc].dp.dt, scenes[sc].dp.grid);
    pos_s[s] = p;
    sceneOfSlot[s] = sc;
}

template <class T>
bool dalloc(T** p, size_t count) {
    if (count == 0) count = 1;
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * count) == cudaSuccess;
}

int from_cuda(cudaError_t e) {
    if (e == cudaSuccess) return PBF_OK;
    if (e == cudaErrorMemoryAllocation) return PBF_ERR_OOM;
    return PBF_ERR_CUDA;
}

int3 dims_of(const sim::GridBounds& g) {
    const float cs = (g.cellSize > 0.f) ? g.cellSize : 1.f;
    int3 d;
    d.x = std::max(0, int(ceilf((g.maxs.x - g.mins.x) / cs)));
    d.y = std::max(0, int(ceilf((g.maxs.y - g.mins.y) / cs)));
    d.z = std::max(0, int(ceilf((g.maxs.z - g.mins.z) / cs)));
    return d;
}

}  // namespace
}  // namespace pbf

struct pbf_ensemble {
    cudaStream_t stream = nullptr;  // where work is enqueued: `own` or a caller's stream
    cudaStream_t own = nullptr;     // created with the ensemble; the graph is captured here
    uint32_t N = 0, S = 0, totalCells = 0;
    int keyBits = 1, passes = 1;
    std::vector<uint32_t> offsets;
    float4 *pos = nullptr, *vel = nullptr, *pred_a = nullptr, *pred_b = nullptr, *pos_s = nullptr, *vel_s = nullptr;
    float* lam = nullptr;
    uint32_t *keys = nullptr, *key_s = nullptr, *perm = nullptr, *lb = nullptr, *sceneOfId = nullptr,
             *sceneOfSlot = nullptr, *err = nullptr, *nbrList = nullptr, *nbrCount = nullptr, *nbrStats = nullptr;
    uint4* tilePlans = nullptr;  // the list build's tile plans (fused_tile_plan_bytes)
    uint32_t nbrCap = 0;
    int tile = 0;  // tile shape of the list passes
    bool fast = false;  // arithmetic of the delta pass (PBF_MATH_FAST)
    pbf::SceneInfo* scenes = nullptr;
    void* sortTemp = nullptr;
    size_t sortBytes = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;

    ~pbf_ensemble() {
        if (stream) cudaStreamSynchronize(stream);
        if (own && own != stream) cudaStreamSynchronize(own);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (void* p : {(void*)pos, (void*)vel, (void*)pred_a, (void*)pred_b, (void*)pos_s, (void*)vel_s, (void*)lam,
                        (void*)keys, (void*)key_s, (void*)perm, (void*)lb, (void*)sceneOfId, (void*)sceneOfSlot,
                        (void*)err, (void*)scenes, sortTemp, (void*)nbrList, (void*)nbrCount, (void*)nbrStats,
                        (void*)tilePlans})
            if (p) cudaFree(p);
        if (own) cudaStreamDestroy(own);
    }

    float4* final_pred() const { return pred_a; }

    pbf::MultiBufs bufs() const {
        pbf::MultiBufs m{};
        m.N = N;
        m.scenes = scenes;
        m.sceneOfSlot = sceneOfSlot;
        m.pos = pos;
        m.vel = vel;
        m.pred_a = pred_a;
        m.pred_b = pred_b;
        m.pos_s = pos_s;
        m.vel_s = vel_s;
        m.lam_s = lam;
        m.key_s = key_s;
        m.perm = perm;
        m.lb = lb;
        m.nbr_list = nbrList;
        m.tile_plans = tilePlans;
        m.nbr_count = nbrCount;
        m.nbr_stats = nbrStats;
        m.nbr_cap = nbrCap;
        m.err = err;
        m.tile = tile;
        m.fast = fast;
        return m;
    }

    // The step as launches on `stream` (captured once into the graph).
    cudaError_t enqueue(cudaStream_t stream) {
        using namespace pbf;
        if (N == 0) return cudaSuccess;
        const unsigned g = blocks_for(N, kBS);
        k_ens_predict_keys<<<g, kBS, 0, stream>>>(pos, vel, scenes, sceneOfId, N, keys);
        cudaError_t e = sort_pairs(sortTemp, sortBytes, keys, key_s, nullptr, perm, N, keyBits, stream, err);
        if (e != cudaSuccess) return e;
        k_ens_gather<<<g, kBS, 0, stream>>>(perm, pos, vel, scenes, sceneOfId, N, pred_a, pos_s, sceneOfSlot);
        if ((e = launch_cell_lb(lb, key_s, N, totalCells, stream)) != cudaSuccess) return e;
        const MultiBufs m = bufs();
        if ((e = multi_build_lists(m, stream)) != cudaSuccess) return e;
        for (int it = 0; it < passes; ++it) {
            if ((e = multi_solve_phase(m, it, 0, stream)) != cudaSuccess) return e;
            if ((e = multi_solve_phase(m, it, 1, stream)) != cudaSuccess) return e;
        }
        return multi_commit(m, final_pred(), stream);
    }

    int capture() {
        if (cudaStreamBeginCapture(own, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return PBF_ERR_CUDA;
        const cudaError_t le = enqueue(own);
        cudaGraph_t gr = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(own, &gr);
        if (le != cudaSuccess || ce != cudaSuccess || !gr) {
            if (gr) cudaGraphDestroy(gr);
            cudaGetLastError();
            return PBF_ERR_CUDA;
        }
        if (cudaGraphInstantiate(&exec, gr, 0) != cudaSuccess) {
            cudaGraphDestroy(gr);
            exec = nullptr;
            return PBF_ERR_CUDA;
        }
        graph = gr;
        return pbf::from_cuda(cudaGraphUpload(exec, stream));
    }

    // Replaces the step graph with one for tile shape `id`.
    int set_tile(int id) {
        if (id == tile && exec) return PBF_OK;
        if (cudaStreamSynchronize(stream) != cudaSuccess) return PBF_ERR_CUDA;
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        tile = id;
        return capture();
    }

    // Replaces the step graph with one for arithmetic mode `f`.
    int set_fast(bool f) {
        if (f == fast && exec) return PBF_OK;
        if (cudaStreamSynchronize(stream) != cudaSuccess) return PBF_ERR_CUDA;
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        fast = f;
        return capture();
    }
};

extern "C" {

int pbf_ensemble_create(const pbf_sim_params* params, uint32_t num_scenes, pbf_ensemble** out) {
    using namespace pbf;
    if (!out) return PBF_ERR_INVALID;
    *out = nullptr;
    if (!params || num_scenes == 0) return PBF_ERR_INVALID;
    const sim::SimParams* sp = reinterpret_cast<const sim::SimParams*>(params);
    std::vector<SceneInfo> info(num_scenes);
    std::vector<uint32_t> offsets(num_scenes + 1, 0);
    uint64_t n = 0, cells = 0;
    int passes = 0;
    for (uint32_t s = 0; s < num_scenes; ++s) {
        sim::SimParams p = sp[s];
        if (p.solverIters < 0 || !(p.grid.cellSize > 0.f)) return PBF_ERR_INVALID;
        p.grid.dim = dims_of(p.grid);
        const uint64_t nc = uint64_t(p.grid.dim.x) * uint64_t(p.grid.dim.y) * uint64_t(p.grid.dim.z);
        if (nc == 0) return PBF_ERR_INVALID;
        std::memset(&info[s], 0, sizeof(SceneInfo));
        info[s].dp = sim::MakeDeviceParams(p);
        info[s].cellOffset = uint32_t(cells);
        info[s].iters = p.solverIters;
        // one list per step where the simulator's schedule builds one
        const int span = list_span_for(p);
        info[s].listUpdates = (span > 0 && span >= p.solverIters) ? p.solverIters : -1;
        offsets[s] = uint32_t(n);
        n += p.numParticles;
        cells += nc;
        passes = std::max(passes, p.solverIters);
        if (n > 0xFFFFFFF0ull || cells > 0xFFFFFFF0ull) return PBF_ERR_UNSUPPORTED;
    }
    offsets[num_scenes] = uint32_t(n);
    pbf_ensemble* e = new (std::nothrow) pbf_ensemble;
    if (!e) return PBF_ERR_OOM;
    e->N = uint32_t(n);
    e->S = num_scenes;
    e->totalCells = uint32_t(cells);
    e->keyBits = bits_for(e->totalCells - 1u);
    e->passes = std::max(1, passes);
    e->offsets = offsets;
    e->sortBytes = sort_temp_bytes(e->N, e->keyBits);
    std::vector<uint32_t> sceneOfId(e->N);
    for (uint32_t s = 0; s < num_scenes; ++s)
        std::fill(sceneOfId.begin() + offsets[s], sceneOfId.begin() + offsets[s + 1], s);
    const uint32_t N = e->N;
    bool ok = cudaStreamCreateWithFlags(&e->own, cudaStreamNonBlocking) == cudaSuccess && dalloc(&e->pos, N) &&
              dalloc(&e->vel, N) && dalloc(&e->pred_a, N) && dalloc(&e->pred_b, N) && dalloc(&e->pos_s, N) &&
              dalloc(&e->vel_s, N) && dalloc(&e->lam, N) && dalloc(&e->keys, N) && dalloc(&e->key_s, N) &&
              dalloc(&e->perm, N) && dalloc(&e->lb, size_t(e->totalCells) + 1) && dalloc(&e->sceneOfId, N) &&
              dalloc(&e->sceneOfSlot, N) && dalloc(&e->err, 1) && dalloc(&e->scenes, num_scenes) &&
              cudaMalloc(&e->sortTemp, e->sortBytes) == cudaSuccess && dalloc(&e->nbrStats, 2) &&
              fused_prepare_kernels() == cudaSuccess;
    e->stream = e->own;
    if (ok) {  // neighbour lists: optional (without them every scene walks the stencil)
        const uint32_t cap = sim::Simulator::kDefaultListCapacity;
        // whole groups of 32 slots: staged tiles interleave the lists of a group
        if (dalloc(&e->nbrList, size_t((uint64_t(N) + 31u) & ~uint64_t(31)) * cap) && dalloc(&e->nbrCount, N) &&
            dalloc(&e->tilePlans, pbf::fused_tile_plan_bytes(N) / sizeof(uint4))) {
            e->nbrCap = cap;
        } else {
            cudaGetLastError();
            if (e->nbrList) cudaFree(e->nbrList);
            e->nbrList = nullptr;
        }
        cudaMemset(e->nbrStats, 0, 2 * sizeof(uint32_t));
    }
    if (ok) {
        ok = cudaMemcpy(e->scenes, info.data(), sizeof(SceneInfo) * num_scenes, cudaMemcpyHostToDevice) ==
                 cudaSuccess &&
             cudaMemcpy(e->sceneOfId, sceneOfId.data(), sizeof(uint32_t) * N, cudaMemcpyHostToDevice) ==
                 cudaSuccess &&
             cudaMemset(e->pos, 0, sizeof(float4) * std::max<uint32_t>(N, 1)) == cudaSuccess &&
             cudaMemset(e->vel, 0, sizeof(float4) * std::max<uint32_t>(N, 1)) == cudaSuccess &&
             cudaMemset(e->err, 0, sizeof(uint32_t)) == cudaSuccess &&
             // legacy-stream copies and clears, finished before the ensemble's
             // non-blocking stream runs
             cudaDeviceSynchronize() == cudaSuccess;
    }
    if (!ok) {
        const cudaError_t ce = cudaGetLastError();
        delete e;
        return ce == cudaErrorMemoryAllocation ? PBF_ERR_OOM : PBF_ERR_CUDA;
    }
    const int st = e->capture();
    if (st != PBF_OK) {
        delete e;
        return st;
    }
    *out = e;
    return PBF_OK;
}

int pbf_ensemble_destroy(pbf_ensemble* e) {
    delete e;
    return PBF_OK;
}

void* pbf_ensemble_stream(pbf_ensemble* e) { return e ? static_cast<void*>(e->stream) : nullptr; }

int pbf_ensemble_set_stream(pbf_ensemble* e, void* stream) {
    if (!e || !e->own) return PBF_ERR_INVALID;
    const cudaStream_t next = stream ? static_cast<cudaStream_t>(stream) : e->own;
    if (next == e->stream) return PBF_OK;
    if (cudaStreamSynchronize(e->stream) != cudaSuccess) return PBF_ERR_CUDA;
    e->stream = next;
    return PBF_OK;
}

uint32_t pbf_ensemble_num_particles(pbf_ensemble* e) { return e ? e->N : 0u; }

int pbf_ensemble_scene_offsets(pbf_ensemble* e, uint32_t* offsets) {
    if (!e || !offsets) return PBF_ERR_INVALID;
    std::memcpy(offsets, e->offsets.data(), sizeof(uint32_t) * e->offsets.size());
    return PBF_OK;
}

int pbf_ensemble_upload_state(pbf_ensemble* e, const float4* pos, const float4* vel) {
    if (!e || !pos || !vel) return PBF_ERR_INVALID;
    const size_t bytes = sizeof(float4) * e->N;
    cudaMemcpyAsync(e->pos, pos, bytes, cudaMemcpyHostToDevice, e->stream);
    cudaMemcpyAsync(e->vel, vel, bytes, cudaMemcpyHostToDevice, e->stream);
    return pbf::from_cuda(cudaStreamSynchronize(e->stream));
}

int pbf_ensemble_download_state(pbf_ensemble* e, float4* pos, float4* vel) {
    if (!e) return PBF_ERR_INVALID;
    const size_t bytes = sizeof(float4) * e->N;
    if (pos) cudaMemcpyAsync(pos, e->pos, bytes, cudaMemcpyDeviceToHost, e->stream);
    if (vel) cudaMemcpyAsync(vel, e->vel, bytes, cudaMemcpyDeviceToHost, e->stream);
    return pbf::from_cuda(cudaStreamSynchronize(e->stream));
}

int pbf_ensemble_step(pbf_ensemble* e, int n) {
    if (!e || n < 0) return PBF_ERR_INVALID;
    for (int i = 0; i < n; ++i)
        if (cudaGraphLaunch(e->exec, e->stream) != cudaSuccess) return PBF_ERR_CUDA;
    return PBF_OK;
}

int pbf_ensemble_step_host(pbf_ensemble* e, float4* pos, float4* vel) {
    if (!e || !pos || !vel) return PBF_ERR_INVALID;
    const size_t bytes = sizeof(float4) * e->N;
    cudaError_t ce = cudaMemcpyAsync(e->pos, pos, bytes, cudaMemcpyHostToDevice, e->stream);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(e->vel, vel, bytes, cudaMemcpyHostToDevice, e->stream);
    if (ce == cudaSuccess) ce = cudaGraphLaunch(e->exec, e->stream);
    if (ce != cudaSuccess) return pbf::from_cuda(ce);
    ce = cudaMemcpyAsync(pos, e->pos, bytes, cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(vel, e->vel, bytes, cudaMemcpyDeviceToHost, e->stream);
    const cudaError_t se = cudaStreamSynchronize(e->stream);
    return pbf::from_cuda(ce != cudaSuccess ? ce : se);
}

int pbf_ensemble_synchronize(pbf_ensemble* e) {
    if (!e) return PBF_ERR_INVALID;
    const cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return pbf::from_cuda(ce);
    uint32_t err = 0;
    if (cudaMemcpy(&err, e->err, sizeof(err), cudaMemcpyDeviceToHost) != cudaSuccess) return PBF_ERR_CUDA;
    if (err) {
        // on the ensemble's stream, so the clear is ordered before its next step
        if (cudaMemsetAsync(e->err, 0, sizeof(uint32_t), e->stream) != cudaSuccess) return PBF_ERR_CUDA;
        if (err & pbf::kErrTimeoutBits) return PBF_ERR_TIMEOUT;
        return (err & pbf::kErrNonFiniteBit) ? PBF_ERR_NONFINITE : PBF_ERR_CUDA;
    }
    return PBF_OK;
}

int pbf_ensemble_set_tile_shape(pbf_ensemble* e, int id) {
    if (!e || id < 0 || id >= pbf::fused_tile_shape_count()) return PBF_ERR_INVALID;
    return e->set_tile(id);
}

int pbf_ensemble_set_math_mode(pbf_ensemble* e, int mode) {
    if (!e || (mode != PBF_MATH_EXACT && mode != PBF_MATH_FAST)) return PBF_ERR_INVALID;
    return e->set_fast(mode == PBF_MATH_FAST);
}

int pbf_ensemble_get_math_mode(pbf_ensemble* e, int* mode) {
    if (!e || !mode) return PBF_ERR_INVALID;
    *mode = e->fast ? PBF_MATH_FAST : PBF_MATH_EXACT;
    return PBF_OK;
}

int pbf_ensemble_get_tile_shape(pbf_ensemble* e, int* id) {
    if (!e || !id) return PBF_ERR_INVALID;
    *id = e->tile;
    return PBF_OK;
}

// Every shape is timed from the same state (one untimed step first, which
// also loads the graph); the state is put back afterwards.
int pbf_ensemble_autotune(pbf_ensemble* e, int steps, float* ms, int* chosen) {
    if (!e || steps < 1) return PBF_ERR_INVALID;
    const int shapes = pbf::fused_tile_shape_count();
    const int before = e->tile;
    const size_t bytes = sizeof(float4) * size_t(e->N);
    float4* snap = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int st = PBF_OK;
    if (cudaStreamSynchronize(e->stream) != cudaSuccess ||
        cudaMalloc(&snap, 2 * std::max<size_t>(bytes, 16)) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess ||
        cudaMemcpyAsync(snap, e->pos, bytes, cudaMemcpyDeviceToDevice, e->stream) != cudaSuccess ||
        cudaMemcpyAsync(snap + e->N, e->vel, bytes, cudaMemcpyDeviceToDevice, e->stream) != cudaSuccess)
        st = PBF_ERR_CUDA;
    auto restore = [&]() {
        return cudaMemcpyAsync(e->pos, snap, bytes, cudaMemcpyDeviceToDevice, e->stream) == cudaSuccess &&
               cudaMemcpyAsync(e->vel, snap + e->N, bytes, cudaMemcpyDeviceToDevice, e->stream) == cudaSuccess;
    };
    std::vector<float> times(size_t(shapes), 0.f);
    for (int id = 0; st == PBF_OK && id < shapes; ++id) {
        if ((st = e->set_tile(id)) != PBF_OK) break;
        bool ok = cudaGraphLaunch(e->exec, e->stream) == cudaSuccess && restore() &&
                  cudaEventRecord(e0, e->stream) == cudaSuccess;
        for (int i = 0; ok && i < steps; ++i) ok = cudaGraphLaunch(e->exec, e->stream) == cudaSuccess;
        float t = 0.f;
        ok = ok && cudaEventRecord(e1, e->stream) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
             cudaEventElapsedTime(&t, e0, e1) == cudaSuccess && restore();
        if (!ok) {
            st = PBF_ERR_CUDA;
            break;
        }
        times[size_t(id)] = t / float(steps);
        if (ms) ms[id] = times[size_t(id)];
    }
    const int best = (st == PBF_OK) ? pbf::pick_tile_shape(times.data(), shapes, before) : before;
    if (snap && !(restore() && cudaStreamSynchronize(e->stream) == cudaSuccess) && st == PBF_OK) st = PBF_ERR_CUDA;
    const int st2 = e->set_tile(st == PBF_OK ? best : before);
    if (st == PBF_OK) st = st2;
    if (e->nbrStats) cudaMemsetAsync(e->nbrStats, 0, 2 * sizeof(uint32_t), e->stream);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (snap) cudaFree(snap);
    if (st == PBF_OK && chosen) *chosen = e->tile;
    return st;
}

int pbf_ensemble_launches_per_step(pbf_ensemble* e) {
    if (!e) return 0;
    const int sortPasses = (e->keyBits + 7) / 8;
    return 1 /*predict_keys*/ + 1 /*hist*/ + sortPasses + 1 /*gather*/ + (e->N > 0 ? 2 : 1) /*lb mark, fill*/ +
           (e->nbrCap ? 1 : 0) /*lists*/ +
           2 * e->passes + 1 /*commit*/;
}

}  // extern "C"
