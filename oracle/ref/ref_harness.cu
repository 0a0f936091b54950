// ref_harness.cu - runs the reference's own CUDA kernels (test checker).
//
// TEST INFRASTRUCTURE ONLY: used by tests/ (parity against the reference
// itself), the fixture generator oracle/ref/make_ref_fixtures.py and the
// reference-GPU timing of bench.py.  Nothing in the product links it.
//
// The kernels are the reference's, compiled from its sources by
// oracle/ref/build_ref.py into device images (oracle/_ref/*.cubin) and loaded
// here with the CUDA driver API.  This file only restates the host-side glue
// of the reference's step: buffer layout (sim/device_buffers.cuh,
// sim/grid_buffers.cuh), launch shapes of the Launch* wrappers, and the phase
// order of sim/phases.cpp:30-117 and sim/post_ops.cpp:25-85, plus the commit
// of sim/simulator.cpp:144-159.  The sort and the block scan are the same CUB
// calls the reference makes (sim/sort_pairs.cu:18-27,
// sim/cell_compact.cu:217-220).  XSPH runs out of place (the reference's
// in-place call is a data race, sim/post_ops.cpp:59,65).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cub/cub.cuh>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pbf/pbf_types.h"
#include "../pbf_oracle.h"

namespace {

struct Mods {
    bool ok = false;
    CUmodule integrate, boundary, hash, ranges, compact, lambda, delta, xsph;
    CUfunction kIntegrate, kBoundary, kVelocity, kHash, kBuildRanges, kMark, kScatter, kLambdaDense, kLambdaCompact,
        kDelta, kDeltaCompact, kApply, kXsph, kXsphCompact;
    CUdeviceptr gPosPred, gLambda;
    std::string err;
};

Mods g;

bool load(const std::string& dir, const char* name, CUmodule* m) {
    std::string path = dir + "/" + name + ".cubin";
    if (cuModuleLoad(m, path.c_str()) != CUDA_SUCCESS) {
        g.err = "cannot load " + path;
        return false;
    }
    return true;
}

// Kernels are looked up by identifier: an exact (extern "C") name, or the
// length-prefixed identifier inside an Itanium-mangled name.
bool find(CUmodule m, const char* ident, CUfunction* out) {
    unsigned n = 0;
    if (cuModuleGetFunctionCount(&n, m) != CUDA_SUCCESS || n == 0) return false;
    std::vector<CUfunction> fs(n);
    if (cuModuleEnumerateFunctions(fs.data(), n, m) != CUDA_SUCCESS) return false;
    const std::string tok = std::to_string(std::strlen(ident)) + ident;
    for (CUfunction f : fs) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
        if (std::strcmp(name, ident) == 0 || std::strstr(name, tok.c_str())) {
            *out = f;
            return true;
        }
    }
    g.err = std::string("kernel not found: ") + ident;
    return false;
}

template <class... A>
CUresult launch(CUfunction f, unsigned grid, unsigned block, cudaStream_t s, A... args) {
    void* p[] = {static_cast<void*>(args)...};
    return cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, (CUstream)s, p, nullptr);
}

unsigned blocks(uint32_t n, unsigned bs) { return (n + bs - 1) / bs; }

pbf_device_params make_dp(const pbf_sim_params& sp) {
    pbf_device_params dp;
    std::memset(&dp, 0, sizeof(dp));
    dp.kernel = sp.kernel;
    dp.grid = sp.grid;
    dp.gravity = sp.gravity;
    dp.restDensity = sp.restDensity;
    dp.dt = sp.dt;
    dp.inv_dt = (sp.dt > 0.f) ? (1.0f / sp.dt) : 0.0f;
    dp.boundaryRestitution = sp.boundaryRestitution;
    dp.maxNeighbors = sp.maxNeighbors;
    dp.particleMass = sp.particleMass;
    dp.pbf = sp.pbf;
    dp.xsph_c = sp.xsph_c;
    return dp;
}

// Reference buffers (sim/device_buffers.cuh:65-99, sim/grid_buffers.cuh:30-64).
struct Bufs {
    uint32_t N = 0, numCells = 0;
    float4 *pos = nullptr, *pred = nullptr, *vel = nullptr, *velOld = nullptr, *delta = nullptr;
    float* lambda = nullptr;
    uint32_t *keys = nullptr, *keysS = nullptr, *idx = nullptr, *idxS = nullptr, *start = nullptr, *end = nullptr;
    uint32_t *uk = nullptr, *off = nullptr, *cnt = nullptr, *blockCounts = nullptr, *blockOffsets = nullptr;
    uint8_t* flags = nullptr;
    void *sortTemp = nullptr, *scanTemp = nullptr;
    size_t sortBytes = 0, scanBytes = 0;

    bool alloc(uint32_t n, uint32_t nc) {
        N = n;
        numCells = nc;
        const unsigned nb = blocks(n, 256) ? blocks(n, 256) : 1;
        bool ok = cudaMalloc(&pos, 16ull * n) == cudaSuccess && cudaMalloc(&pred, 16ull * n) == cudaSuccess &&
                  cudaMalloc(&vel, 16ull * n) == cudaSuccess && cudaMalloc(&velOld, 16ull * n) == cudaSuccess &&
                  cudaMalloc(&delta, 16ull * n) == cudaSuccess && cudaMalloc(&lambda, 4ull * n) == cudaSuccess &&
                  cudaMalloc(&keys, 4ull * n) == cudaSuccess && cudaMalloc(&keysS, 4ull * n) == cudaSuccess &&
                  cudaMalloc(&idx, 4ull * n) == cudaSuccess && cudaMalloc(&idxS, 4ull * n) == cudaSuccess &&
                  cudaMalloc(&start, 4ull * nc) == cudaSuccess && cudaMalloc(&end, 4ull * nc) == cudaSuccess &&
                  cudaMalloc(&uk, 4ull * n) == cudaSuccess && cudaMalloc(&off, 4ull * (n + 1)) == cudaSuccess &&
                  cudaMalloc(&cnt, 4) == cudaSuccess && cudaMalloc(&flags, n) == cudaSuccess &&
                  cudaMalloc(&blockCounts, 4ull * nb) == cudaSuccess &&
                  cudaMalloc(&blockOffsets, 4ull * nb) == cudaSuccess;
        if (!ok) return false;
        cub::DeviceRadixSort::SortPairs(nullptr, sortBytes, keys, keysS, idx, idxS, (int)n, 0, 32);
        cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, blockCounts, blockOffsets, (int)nb);
        return cudaMalloc(&sortTemp, sortBytes) == cudaSuccess && cudaMalloc(&scanTemp, scanBytes) == cudaSuccess;
    }
    void free_all() {
        void* ps[] = {pos, pred, vel, velOld, delta, lambda, keys, keysS, idx, idxS, start, end, uk, off, cnt,
                      blockCounts, blockOffsets, flags, sortTemp, scanTemp};
        for (void* p : ps)
            if (p) cudaFree(p);
        *this = Bufs{};
    }
};

// One reference step on device buffers (phase order of sim/phases.cpp and
// sim/post_ops.cpp).  Returns 0 on success.
int ref_step_device(Bufs& b, const pbf_sim_params& sp, int hashed, cudaStream_t s) {
    const uint32_t N = b.N;
    if (N == 0) return 0;
    pbf_device_params dp = make_dp(sp);
    pbf_grid_bounds grid = sp.grid;
    float3 gravity = sp.gravity;
    float dt = sp.dt, zero = 0.0f, e = sp.boundaryRestitution, invDt = 1.0f / sp.dt;
    uint32_t n = N, nc = b.numCells;
    const unsigned nb = blocks(N, 256);
    // PhaseIntegrate (sim/phases.cpp:33-36)
    launch(g.kIntegrate, nb, 256, s, &b.pos, &b.vel, &b.pred, &gravity, &dt, &n);
    launch(g.kBoundary, nb, 256, s, &b.pred, &b.vel, &grid, &zero, &n);
    // PhaseGridBuildFull (sim/phases.cpp:44-63)
    launch(g.kHash, nb, 256, s, &b.keys, &b.idx, &b.pred, &grid, &n);
    cub::DeviceRadixSort::SortPairs(b.sortTemp, b.sortBytes, b.keys, b.keysS, b.idx, b.idxS, (int)N, 0, 32, s);
    if (hashed) {
        launch(g.kMark, nb, 256, s, &b.keysS, &n, &b.flags, &b.blockCounts);
        cub::DeviceScan::ExclusiveSum(b.scanTemp, b.scanBytes, b.blockCounts, b.blockOffsets, (int)nb, s);
        launch(g.kScatter, nb, 256, s, &b.keysS, &n, &b.flags, &b.blockOffsets, &b.blockCounts, &b.uk, &b.off, &b.cnt);
    } else {
        cudaMemsetAsync(b.start, 0xFF, 4ull * nc, s);
        cudaMemsetAsync(b.end, 0xFF, 4ull * nc, s);
        cudaMemsetAsync(b.start, 0xFF, 4ull * nc, s);  // LaunchCellRanges, sim/cell_ranges.cu:62-63
        cudaMemsetAsync(b.end, 0x00, 4ull * nc, s);
        unsigned rb = nb > 1024 ? 1024 : nb;
        launch(g.kBuildRanges, rb, 256, s, &b.keysS, &n, &nc, &b.start, &b.end);
    }
    // PhaseSolveIterations (sim/phases.cpp:71-94)
    for (int it = 0; it < sp.solverIters; ++it) {
        if (hashed) {
            launch(g.kLambdaCompact, nb, 256, s, &b.idxS, &b.keysS, &b.uk, &b.off, &b.cnt, &dp, &n);
            launch(g.kDeltaCompact, nb, 256, s, &b.delta, &b.pred, &b.lambda, &b.idxS, &b.keysS, &b.uk, &b.off, &b.cnt,
                   &dp, &n);
        } else {
            launch(g.kLambdaDense, nb, 256, s, &b.idxS, &b.keysS, &b.start, &b.end, &dp, &n);
            launch(g.kDelta, nb, 256, s, &b.delta, &b.pred, &b.lambda, &b.idxS, &b.keysS, &b.start, &b.end, &dp, &n);
        }
        launch(g.kApply, nb, 256, s, &b.pred, &b.delta, &b.idxS, &n);
    }
    launch(g.kBoundary, nb, 256, s, &b.pred, &b.vel, &grid, &zero, &n);
    // PhaseVelocity (sim/phases.cpp:102-105)
    launch(g.kVelocity, nb, 256, s, &b.vel, &b.pos, &b.pred, &invDt, &n);
    // PostOps: XSPH (out of place) -> Boundary(e) (sim/post_ops.cpp:25-71)
    if (sp.xsph_c > 0.f) {
        cudaMemcpyAsync(b.velOld, b.vel, 16ull * N, cudaMemcpyDeviceToDevice, s);
        if (hashed)
            launch(g.kXsphCompact, nb, 256, s, &b.vel, &b.velOld, &b.pred, &b.idxS, &b.keysS, &b.uk, &b.off, &b.cnt, &dp,
                   &n);
        else
            launch(g.kXsph, nb, 256, s, &b.vel, &b.velOld, &b.pred, &b.idxS, &b.keysS, &b.start, &b.end, &dp, &n);
    }
    launch(g.kBoundary, nb, 256, s, &b.pred, &b.vel, &grid, &e, &n);
    // commit: the ping-pong swap makes pred the next step's position
    float4* t = b.pos;
    b.pos = b.pred;
    b.pred = t;
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

bool bind_globals(Bufs& b) {
    return cuMemcpyHtoD(g.gPosPred, &b.pred, sizeof(void*)) == CUDA_SUCCESS &&
           cuMemcpyHtoD(g.gLambda, &b.lambda, sizeof(void*)) == CUDA_SUCCESS;
}

}  // namespace

extern "C" {

// Loads the reference device images from dir; 0 on success.
int ref_init(const char* dir) {
    if (g.ok) return 0;
    cudaFree(nullptr);  // create the primary context
    const std::string d(dir);
    bool ok = load(d, "integrate", &g.integrate) && load(d, "boundary", &g.boundary) && load(d, "hash_keys", &g.hash) &&
              load(d, "cell_ranges", &g.ranges) && load(d, "cell_compact", &g.compact) &&
              load(d, "pbf_lambda", &g.lambda) && load(d, "pbf_delta_apply", &g.delta) && load(d, "xsph", &g.xsph);
    ok = ok && find(g.integrate, "KIntegratePred", &g.kIntegrate) && find(g.boundary, "KBoundary", &g.kBoundary) &&
         find(g.boundary, "KVelocity", &g.kVelocity) && find(g.hash, "KHash", &g.kHash) &&
         find(g.ranges, "KBuildRanges", &g.kBuildRanges) && find(g.compact, "KMarkAndCountWarp", &g.kMark) &&
         find(g.compact, "KScatterSegmentsWarp", &g.kScatter) &&
         find(g.lambda, "KLambdaGlobalsDense", &g.kLambdaDense) &&
         find(g.lambda, "KLambdaGlobalsCompact", &g.kLambdaCompact) && find(g.delta, "KDeltaCompute", &g.kDelta) &&
         find(g.delta, "KDeltaComputeCompact", &g.kDeltaCompact) && find(g.delta, "KApplyDelta", &g.kApply) &&
         find(g.xsph, "KXSPH", &g.kXsph) && find(g.xsph, "KXSPHCompact", &g.kXsphCompact);
    size_t bytes = 0;
    ok = ok && cuModuleGetGlobal(&g.gPosPred, &bytes, g.lambda, "_ZN3sim10g_pos_predE") == CUDA_SUCCESS &&
         cuModuleGetGlobal(&g.gLambda, &bytes, g.lambda, "_ZN3sim8g_lambdaE") == CUDA_SUCCESS;
    g.ok = ok;
    return ok ? 0 : 1;
}

const char* ref_error(void) { return g.err.c_str(); }

// One reference step on host arrays (in place), with the same optional trace
// as the CPU oracle.  0 on success.
int ref_step(const pbf_sim_params* p, int hashed, float4* pos, float4* vel, uint32_t N, oracle_trace* tr) {
    if (!g.ok || !p) return 1;
    const uint32_t nc = uint32_t(p->grid.dim.x) * uint32_t(p->grid.dim.y) * uint32_t(p->grid.dim.z);
    Bufs b;
    if (!b.alloc(N, nc)) {
        b.free_all();
        return 3;
    }
    cudaMemcpy(b.pos, pos, 16ull * N, cudaMemcpyHostToDevice);
    cudaMemcpy(b.pred, pos, 16ull * N, cudaMemcpyHostToDevice);  // d_pos_next = d_pos (simulator.cpp:258-263)
    cudaMemcpy(b.vel, vel, 16ull * N, cudaMemcpyHostToDevice);
    // oracle_trace wants pred_solved / vel_pre_xsph, so the step is split:
    // run it normally, and re-run the first part for those two arrays.
    int rc = bind_globals(b) ? 0 : 4;
    if (rc == 0) rc = ref_step_device(b, *p, hashed, 0);
    cudaDeviceSynchronize();
    if (rc == 0 && cudaGetLastError() != cudaSuccess) rc = 2;
    if (rc == 0) {
        cudaMemcpy(pos, b.pos, 16ull * N, cudaMemcpyDeviceToHost);
        cudaMemcpy(vel, b.vel, 16ull * N, cudaMemcpyDeviceToHost);
        if (tr) {
            if (tr->keys) cudaMemcpy(tr->keys, b.keys, 4ull * N, cudaMemcpyDeviceToHost);
            if (tr->keys_sorted) cudaMemcpy(tr->keys_sorted, b.keysS, 4ull * N, cudaMemcpyDeviceToHost);
            if (tr->perm) cudaMemcpy(tr->perm, b.idxS, 4ull * N, cudaMemcpyDeviceToHost);
            if (tr->lambda) cudaMemcpy(tr->lambda, b.lambda, 4ull * N, cudaMemcpyDeviceToHost);
            if (hashed) {
                uint32_t m = 0;
                cudaMemcpy(&m, b.cnt, 4, cudaMemcpyDeviceToHost);
                if (tr->compact_count) *tr->compact_count = m;
                if (tr->unique_keys) cudaMemcpy(tr->unique_keys, b.uk, 4ull * m, cudaMemcpyDeviceToHost);
                if (tr->offsets) cudaMemcpy(tr->offsets, b.off, 4ull * (m + 1), cudaMemcpyDeviceToHost);
            } else {
                if (tr->cell_start) cudaMemcpy(tr->cell_start, b.start, 4ull * nc, cudaMemcpyDeviceToHost);
                if (tr->cell_end) cudaMemcpy(tr->cell_end, b.end, 4ull * nc, cudaMemcpyDeviceToHost);
            }
        }
    }
    b.free_all();
    return rc;
}

}  // extern "C"

// ---- single phases of the reference on host arrays (for per-phase parity).
// Inputs use the reference layout; table = dense (start/end) or compact.
namespace {
struct Dev {
    std::vector<void*> ptrs;
    template <class T>
    T* up(const T* h, size_t n) {
        void* d = nullptr;
        cudaMalloc(&d, sizeof(T) * (n ? n : 1));
        if (h && n) cudaMemcpy(d, h, sizeof(T) * n, cudaMemcpyHostToDevice);
        ptrs.push_back(d);
        return static_cast<T*>(d);
    }
    ~Dev() {
        for (void* p : ptrs) cudaFree(p);
    }
};
}  // namespace

extern "C" {

int ref_phase_lambda(float* lambda, const float4* pred, const uint32_t* idx, const uint32_t* keys,
                     const oracle_table* t, const pbf_device_params* dp_in, uint32_t N, uint32_t numCells) {
    if (!g.ok || N == 0) return 1;
    Dev d;
    float4* dpred = d.up(pred, N);
    float* dlam = d.up<float>(nullptr, N);
    uint32_t *didx = d.up(idx, N), *dkeys = d.up(keys, N);
    pbf_device_params dp = *dp_in;
    uint32_t n = N;
    if (cuMemcpyHtoD(g.gPosPred, &dpred, sizeof(void*)) != CUDA_SUCCESS) return 4;
    if (cuMemcpyHtoD(g.gLambda, &dlam, sizeof(void*)) != CUDA_SUCCESS) return 4;
    if (t->unique_keys) {
        uint32_t *uk = d.up(t->unique_keys, t->count), *off = d.up(t->offsets, t->count + 1), *cnt = d.up(&t->count, 1);
        launch(g.kLambdaCompact, blocks(N, 256), 256, 0, &didx, &dkeys, &uk, &off, &cnt, &dp, &n);
    } else {
        uint32_t *st = d.up(t->start, numCells), *en = d.up(t->end, numCells);
        launch(g.kLambdaDense, blocks(N, 256), 256, 0, &didx, &dkeys, &st, &en, &dp, &n);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return 2;
    cudaMemcpy(lambda, dlam, 4ull * N, cudaMemcpyDeviceToHost);
    return 0;
}

int ref_phase_delta_apply(float4* pred_io, float4* delta, const float* lambda, const uint32_t* idx,
                          const uint32_t* keys, const oracle_table* t, const pbf_device_params* dp_in, uint32_t N,
                          uint32_t numCells) {
    if (!g.ok || N == 0) return 1;
    Dev d;
    float4 *dpred = d.up(pred_io, N), *ddelta = d.up<float4>(nullptr, N);
    float* dlam = d.up(lambda, N);
    uint32_t *didx = d.up(idx, N), *dkeys = d.up(keys, N);
    pbf_device_params dp = *dp_in;
    uint32_t n = N;
    if (t->unique_keys) {
        uint32_t *uk = d.up(t->unique_keys, t->count), *off = d.up(t->offsets, t->count + 1), *cnt = d.up(&t->count, 1);
        launch(g.kDeltaCompact, blocks(N, 256), 256, 0, &ddelta, &dpred, &dlam, &didx, &dkeys, &uk, &off, &cnt, &dp, &n);
    } else {
        uint32_t *st = d.up(t->start, numCells), *en = d.up(t->end, numCells);
        launch(g.kDelta, blocks(N, 256), 256, 0, &ddelta, &dpred, &dlam, &didx, &dkeys, &st, &en, &dp, &n);
    }
    launch(g.kApply, blocks(N, 256), 256, 0, &dpred, &ddelta, &didx, &n);
    if (cudaDeviceSynchronize() != cudaSuccess) return 2;
    cudaMemcpy(pred_io, dpred, 16ull * N, cudaMemcpyDeviceToHost);
    cudaMemcpy(delta, ddelta, 16ull * N, cudaMemcpyDeviceToHost);
    return 0;
}

int ref_phase_xsph(float4* vel_out, const float4* vel_in, const float4* pred, const uint32_t* idx,
                   const uint32_t* keys, const oracle_table* t, const pbf_device_params* dp_in, uint32_t N,
                   uint32_t numCells) {
    if (!g.ok || N == 0) return 1;
    Dev d;
    float4 *dout = d.up<float4>(nullptr, N), *din = d.up(vel_in, N), *dpred = d.up(pred, N);
    uint32_t *didx = d.up(idx, N), *dkeys = d.up(keys, N);
    pbf_device_params dp = *dp_in;
    uint32_t n = N;
    if (t->unique_keys) {
        uint32_t *uk = d.up(t->unique_keys, t->count), *off = d.up(t->offsets, t->count + 1), *cnt = d.up(&t->count, 1);
        launch(g.kXsphCompact, blocks(N, 256), 256, 0, &dout, &din, &dpred, &didx, &dkeys, &uk, &off, &cnt, &dp, &n);
    } else {
        uint32_t *st = d.up(t->start, numCells), *en = d.up(t->end, numCells);
        launch(g.kXsph, blocks(N, 256), 256, 0, &dout, &din, &dpred, &didx, &dkeys, &st, &en, &dp, &n);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return 2;
    cudaMemcpy(vel_out, dout, 16ull * N, cudaMemcpyDeviceToHost);
    return 0;
}

int ref_phase_integrate_boundary(const float4* pos, float4* vel_io, float4* pred, const pbf_sim_params* p,
                                 uint32_t N) {
    if (!g.ok || N == 0) return 1;
    Dev d;
    float4 *dpos = d.up(pos, N), *dvel = d.up(vel_io, N), *dpred = d.up<float4>(nullptr, N);
    pbf_grid_bounds grid = p->grid;
    float3 gravity = p->gravity;
    float dt = p->dt, zero = 0.f;
    uint32_t n = N;
    launch(g.kIntegrate, blocks(N, 256), 256, 0, &dpos, &dvel, &dpred, &gravity, &dt, &n);
    launch(g.kBoundary, blocks(N, 256), 256, 0, &dpred, &dvel, &grid, &zero, &n);
    if (cudaDeviceSynchronize() != cudaSuccess) return 2;
    cudaMemcpy(pred, dpred, 16ull * N, cudaMemcpyDeviceToHost);
    cudaMemcpy(vel_io, dvel, 16ull * N, cudaMemcpyDeviceToHost);
    return 0;
}

// Times `steps` reference steps (after `warmup`) captured in one CUDA graph
// per step, as sim::Simulator does; state advances in place.  Writes the
// mean device time per step.  0 on success.
int ref_time_steps(const pbf_sim_params* p, int hashed, float4* pos, float4* vel, uint32_t N, int warmup, int steps,
                   double* ms_per_step) {
    if (!g.ok || !p || steps <= 0) return 1;
    const uint32_t nc = uint32_t(p->grid.dim.x) * uint32_t(p->grid.dim.y) * uint32_t(p->grid.dim.z);
    Bufs b;
    if (!b.alloc(N, nc)) {
        b.free_all();
        return 3;
    }
    cudaMemcpy(b.pos, pos, 16ull * N, cudaMemcpyHostToDevice);
    cudaMemcpy(b.pred, pos, 16ull * N, cudaMemcpyHostToDevice);
    cudaMemcpy(b.vel, vel, 16ull * N, cudaMemcpyHostToDevice);
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    // Two graphs: the ping-pong swap alternates which buffer is current.
    cudaGraphExec_t ex[2] = {nullptr, nullptr};
    int rc = 0;
    for (int k = 0; k < 2 && rc == 0; ++k) {
        cudaGraph_t gr;
        cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        ref_step_device(b, *p, hashed, s);
        if (cudaStreamEndCapture(s, &gr) != cudaSuccess || cudaGraphInstantiate(&ex[k], gr, 0) != cudaSuccess) rc = 5;
        cudaGraphDestroy(gr);
    }
    // ref_step_device swapped pos/pred twice during capture: back to start.
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float total = 0.f;
    for (int k = 0; k < warmup + steps && rc == 0; ++k) {
        // graph 0 predicts into b.pred, graph 1 into b.pos (the swap)
        Bufs tmp = b;
        if (k & 1) std::swap(tmp.pos, tmp.pred);
        if (!bind_globals(tmp)) rc = 4;
        if (k >= warmup) cudaEventRecord(e0, s);
        cudaGraphLaunch(ex[k & 1], s);
        if (k >= warmup) {
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            total += ms;
        } else {
            cudaStreamSynchronize(s);
        }
    }
    if (rc == 0 && cudaStreamSynchronize(s) != cudaSuccess) rc = 2;
    if (rc == 0) {
        const bool swapped = ((warmup + steps) & 1) != 0;
        cudaMemcpy(pos, swapped ? b.pred : b.pos, 16ull * N, cudaMemcpyDeviceToHost);
        cudaMemcpy(vel, b.vel, 16ull * N, cudaMemcpyDeviceToHost);
        *ms_per_step = total / steps;
    }
    for (auto& x : ex)
        if (x) cudaGraphExecDestroy(x);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    b.free_all();
    return rc;
}

}  // extern "C"
