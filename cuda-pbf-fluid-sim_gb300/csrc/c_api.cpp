// c_api.cpp - the extern "C" surface of libpbf_gb300 (include/pbf/pbf.h,
// include/pbf/launch_abi.h).
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "../../include/pbf/launch_abi.h"
#include "../../include/pbf/pbf.h"
#include "../../include/pbf/simulator.h"
#include "fused.cuh"
#include "grid.cuh"
#include "pbf_errors.h"
#include "phases.cuh"
#include "sort.cuh"

#include "handle.h"

namespace {

int from_cuda(cudaError_t e) {
    if (e == cudaSuccess) return PBF_OK;
    if (e == cudaErrorMemoryAllocation) return PBF_ERR_OOM;
    return PBF_ERR_CUDA;
}

int launch_status() { return from_cuda(cudaGetLastError()); }

const sim::GridBounds& G(const pbf_grid_bounds* g) { return *reinterpret_cast<const sim::GridBounds*>(g); }
const sim::DeviceParams& D(const pbf_device_params* d) { return *reinterpret_cast<const sim::DeviceParams*>(d); }
const sim::SimParams& S(const pbf_sim_params* p) { return *reinterpret_cast<const sim::SimParams*>(p); }

// Process-global scratch of the reference-name compact launcher: the
// reference's LaunchCellRangesCompact owns static scratch the same way
// (sim/cell_compact.cu:50-93) and is equally non-re-entrant.
void* g_compactScratch = nullptr;
size_t g_compactScratchBytes = 0;

bool ensure_global_compact_scratch(uint32_t N) {
    const size_t need = pbf::compact_scratch_bytes(N);
    if (need <= g_compactScratchBytes && g_compactScratch) return true;
    if (g_compactScratch) cudaFree(g_compactScratch);
    g_compactScratch = nullptr;
    g_compactScratchBytes = 0;
    if (cudaMalloc(&g_compactScratch, need) != cudaSuccess) return false;
    g_compactScratchBytes = need;
    return true;
}

// std::mt19937_64 draw -> double in [0,1) from its top 53 bits.
inline double unit53(std::mt19937_64& rng) { return double(rng() >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace

extern "C" {

// ------------------------------------------------------------- status
const char* pbf_status_string(int s) {
    switch (s) {
        case PBF_OK: return "ok";
        case PBF_ERR_INVALID: return "invalid argument";
        case PBF_ERR_CUDA: return "CUDA error";
        case PBF_ERR_OOM: return "out of memory";
        case PBF_ERR_TIMEOUT: return "bounded device wait gave up";
        case PBF_ERR_NONFINITE: return "non-finite particle state";
        case PBF_ERR_UNSUPPORTED: return "unsupported";
        default: return "unknown status";
    }
}

int pbf_version(void) { return 10000; }

void pbf_abi_sizes(uint32_t out[5]) {
    if (!out) return;
    out[0] = sizeof(pbf_kernel_coeffs);
    out[1] = sizeof(pbf_grid_bounds);
    out[2] = sizeof(pbf_tuning);
    out[3] = sizeof(pbf_sim_params);
    out[4] = sizeof(pbf_device_params);
}

// ---------------------------------------------------------- parameters
void pbf_default_tuning(pbf_tuning* out) {
    if (!out) return;
    sim::PbfTuning t{};
    std::memcpy(out, &t, sizeof(t));
}

void pbf_make_kernel_coeffs(float h, pbf_kernel_coeffs* out) {
    if (!out) return;
    sim::KernelCoeffs kc = sim::MakeKernelCoeffs(h);
    std::memcpy(out, &kc, sizeof(kc));
}

void pbf_make_device_params(const pbf_sim_params* sp, pbf_device_params* out) {
    if (!sp || !out) return;
    sim::DeviceParams dp = sim::MakeDeviceParams(S(sp));
    std::memcpy(out, &dp, sizeof(dp));
}

void pbf_compute_dims(const pbf_grid_bounds* g, int32_t out_dim[3]) {
    if (!g || !out_dim) return;
    const float cs = (g->cellSize > 0.f) ? g->cellSize : 1.f;
    int d[3] = {int(ceilf((g->maxs.x - g->mins.x) / cs)), int(ceilf((g->maxs.y - g->mins.y) / cs)),
                int(ceilf((g->maxs.z - g->mins.z) / cs))};
    for (int k = 0; k < 3; ++k) out_dim[k] = d[k] < 0 ? 0 : d[k];
}

int pbf_dam_break_params(float bx, float by, float bz, int solver_iters, uint32_t num_particles,
                         pbf_sim_params* out) {
    if (!out || !(bx > 0.f) || !(by > 0.f) || !(bz > 0.f) || solver_iters < 0) return PBF_ERR_INVALID;
    sim::SimParams sp{};
    const float r = 0.005f;
    const float spacing = 0.01f;  // 2r
    const float h = 2.5f * r;     // h_over_r * r (engine/core/console.cpp:219-224)
    sp.numParticles = num_particles;
    sp.maxParticles = num_particles;
    sp.gravity = make_float3(0.0f, -9.8f, 0.0f);
    sp.dt = 1.0f / 120.0f;
    sp.cfl = 0.45f;
    sp.solverIters = solver_iters;
    sp.maxNeighbors = 64;
    sp.sortEveryN = 1;
    sp.boundaryRestitution = 0.0f;
    sp.particleMass = 1000.0f * spacing * spacing * spacing;
    sp.pbf = sim::PbfTuning{};
    sp.pbf.scorr_enable = 1;
    sp.pbf.scorr_k = 0.1f;
    sp.pbf.scorr_n = 4.0f;
    sp.pbf.scorr_dq_h = 0.2f;
    sp.pbf.lambda_denom_eps = 100.0f;
    sp.pbf.compliance = 0.0f;
    sp.pbf.xpbd_enable = 0;
    sp.xsph_c = 0.01f;
    sp.kernel = sim::MakeKernelCoeffs(h);
    // Rest density of an interior particle of the unjittered lattice,
    // accumulated exactly as the lambda kernel does (self term excluded,
    // sim/pbf_lambda.cu:63): the 6 face neighbours at distance `spacing` are
    // the only ones within h (the next shell is at sqrt(2)*spacing > h).
    {
        const sim::KernelCoeffs& kc = sp.kernel;
        float density = 0.f;
        for (int n = 0; n < 6; ++n) {
            const float r2 = spacing * spacing;
            const float hr2 = kc.h2 - r2;
            density += sp.particleMass * kc.poly6 * hr2 * hr2 * hr2;
        }
        sp.restDensity = density;
    }
    sp.grid.mins = make_float3(0.f, 0.f, 0.f);
    sp.grid.maxs = make_float3(bx, by, bz);
    sp.grid.cellSize = std::fmax(1e-6f, 1.0f * h);
    int32_t d[3];
    pbf_compute_dims(reinterpret_cast<const pbf_grid_bounds*>(&sp.grid), d);
    sp.grid.dim = make_int3(d[0] < 1 ? 1 : d[0], d[1] < 1 ? 1 : d[1], d[2] < 1 ? 1 : d[2]);
    sp.ghostParticleCount = 0;
    std::memcpy(out, &sp, sizeof(sp));
    return PBF_OK;
}

int pbf_seed_lattice(float4* pos_out, uint32_t nx, uint32_t ny, uint32_t nz, float ox, float oy, float oz,
                     float spacing, float jitter, uint64_t seed, const pbf_grid_bounds* box) {
    if (!pos_out || !box) return PBF_ERR_INVALID;
    std::mt19937_64 rng(seed);
    const pbf_grid_bounds& g = *box;
    uint64_t id = 0;
    for (uint32_t iz = 0; iz < nz; ++iz)
        for (uint32_t iy = 0; iy < ny; ++iy)
            for (uint32_t ix = 0; ix < nx; ++ix) {
                float x = ox + float(ix) * spacing;
                float y = oy + float(iy) * spacing;
                float z = oz + float(iz) * spacing;
                const float jx = float((2.0 * unit53(rng) - 1.0) * double(jitter));
                const float jy = float((2.0 * unit53(rng) - 1.0) * double(jitter));
                const float jz = float((2.0 * unit53(rng) - 1.0) * double(jitter));
                x = std::fmin(std::fmax(x + jx, g.mins.x), g.maxs.x);
                y = std::fmin(std::fmax(y + jy, g.mins.y), g.maxs.y);
                z = std::fmin(std::fmax(z + jz, g.mins.z), g.maxs.z);
                pos_out[id].x = x;
                pos_out[id].y = y;
                pos_out[id].z = z;
                pos_out[id].w = 1.0f;
                ++id;
            }
    return PBF_OK;
}

// ------------------------------------------------------ phase launchers
int pbf_launch_integrate_pred(const float4* posCurr, const float4* velSrc, float4* posPred, float3 gravity,
                              float dt, uint32_t N, cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!posCurr || !velSrc || !posPred) return PBF_ERR_INVALID;
    return from_cuda(pbf::launch_integrate_pred_ref(posCurr, velSrc, posPred, gravity, dt, N, s));
}

int pbf_launch_boundary(float4* pos_pred, float4* vel, const pbf_grid_bounds* grid, float restitution, uint32_t N,
                        cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!pos_pred || !vel || !grid) return PBF_ERR_INVALID;
    return from_cuda(pbf::launch_boundary_ref(pos_pred, vel, G(grid), restitution, N, s));
}

int pbf_launch_velocity(float4* vel, const float4* pos, const float4* pos_pred, float inv_dt, uint32_t N,
                        cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!vel || !pos || !pos_pred) return PBF_ERR_INVALID;
    return from_cuda(pbf::launch_velocity_ref(vel, pos, pos_pred, inv_dt, N, s));
}

int pbf_launch_hash_keys(uint32_t* keys, uint32_t* indices, const float4* pos, const pbf_grid_bounds* grid,
                         uint32_t N, cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!keys || !indices || !pos || !grid) return PBF_ERR_INVALID;
    if (grid->dim.x <= 0 || grid->dim.y <= 0 || grid->dim.z <= 0) return PBF_ERR_INVALID;
    return from_cuda(pbf::launch_hash_keys_ref(keys, indices, pos, G(grid), N, s));
}

int pbf_sort_pairs_query(size_t* tempBytes, uint32_t N) {
    if (!tempBytes) return PBF_ERR_INVALID;
    *tempBytes = pbf::sort_temp_bytes(N, 32);
    return PBF_OK;
}

int pbf_launch_sort_pairs_bits(void* d_temp, size_t tempBytes, const uint32_t* keys_in, uint32_t* keys_out,
                               const uint32_t* vals_in, uint32_t* vals_out, uint32_t N, int num_bits,
                               cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!keys_in || !keys_out || !vals_in || !vals_out || !d_temp) return PBF_ERR_INVALID;
    if (keys_in == keys_out || vals_in == vals_out || num_bits < 1 || num_bits > 32) return PBF_ERR_INVALID;
    if (tempBytes < pbf::sort_temp_bytes(N, num_bits)) return PBF_ERR_INVALID;
    return from_cuda(pbf::sort_pairs(d_temp, tempBytes, keys_in, keys_out, vals_in, vals_out, N, num_bits, s, nullptr));
}

int pbf_launch_sort_pairs(void* d_temp, size_t tempBytes, const uint32_t* keys_in, uint32_t* keys_out,
                          const uint32_t* vals_in, uint32_t* vals_out, uint32_t N, cudaStream_t s) {
    return pbf_launch_sort_pairs_bits(d_temp, tempBytes, keys_in, keys_out, vals_in, vals_out, N, 32, s);
}

int pbf_launch_cell_ranges(uint32_t* cellStart, uint32_t* cellEnd, const uint32_t* keysSorted, uint32_t N,
                           uint32_t numCells, cudaStream_t s) {
    if (numCells == 0) return PBF_OK;
    if (!cellStart || !cellEnd || (N > 0 && !keysSorted)) return PBF_ERR_INVALID;
    return from_cuda(pbf::launch_cell_ranges_ref(cellStart, cellEnd, keysSorted, N, numCells, s));
}

int pbf_cell_compact_scratch_query(size_t* bytes, uint32_t N) {
    if (!bytes) return PBF_ERR_INVALID;
    *bytes = pbf::compact_scratch_bytes(N);
    return PBF_OK;
}

int pbf_launch_cell_ranges_compact(void* d_scratch, size_t scratchBytes, uint32_t* uniqueKeys, uint32_t* offsets,
                                   uint32_t* compactCount, const uint32_t* keysSorted, uint32_t N, cudaStream_t s) {
    if (!offsets || !compactCount) return PBF_ERR_INVALID;
    if (N > 0 && (!uniqueKeys || !keysSorted || !d_scratch)) return PBF_ERR_INVALID;
    if (N > 0 && scratchBytes < pbf::compact_scratch_bytes(N)) return PBF_ERR_INVALID;
    return from_cuda(pbf::launch_compact(d_scratch, scratchBytes, uniqueKeys, offsets, compactCount, nullptr,
                                         keysSorted, N, s, nullptr));
}

static pbf::RefTable dense_table(const uint32_t* start, const uint32_t* end) {
    return pbf::RefTable{start, end, nullptr, nullptr, nullptr};
}
static pbf::RefTable compact_table(const uint32_t* uk, const uint32_t* off, const uint32_t* cnt) {
    return pbf::RefTable{nullptr, nullptr, uk, off, cnt};
}

static bool valid_dp(const pbf_device_params* dp) {
    return dp && dp->grid.dim.x > 0 && dp->grid.dim.y > 0 && dp->grid.dim.z > 0;
}

int pbf_launch_lambda(float* lambda, const float4* pos_pred, const uint32_t* idx, const uint32_t* keys,
                      const uint32_t* cellStart, const uint32_t* cellEnd, const pbf_device_params* dp, uint32_t N,
                      cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!lambda || !pos_pred || !idx || !keys || !cellStart || !cellEnd || !valid_dp(dp)) return PBF_ERR_INVALID;
    return from_cuda(pbf::launch_lambda_ref(lambda, pos_pred, idx, keys, dense_table(cellStart, cellEnd), D(dp), N, s));
}

int pbf_launch_lambda_compact(float* lambda, const float4* pos_pred, const uint32_t* idx, const uint32_t* keys,
                              const uint32_t* uk, const uint32_t* off, const uint32_t* cnt,
                              const pbf_device_params* dp, uint32_t N, cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!lambda || !pos_pred || !idx || !keys || !uk || !off || !cnt || !valid_dp(dp)) return PBF_ERR_INVALID;
    return from_cuda(pbf::launch_lambda_ref(lambda, pos_pred, idx, keys, compact_table(uk, off, cnt), D(dp), N, s));
}

int pbf_launch_delta_apply(float4* pos_pred, float4* delta, const float* lambda, const uint32_t* idx,
                           const uint32_t* keys, const uint32_t* cellStart, const uint32_t* cellEnd,
                           const pbf_device_params* dp, uint32_t N, cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!pos_pred || !delta || !lambda || !idx || !keys || !cellStart || !cellEnd || !valid_dp(dp))
        return PBF_ERR_INVALID;
    return from_cuda(
        pbf::launch_delta_apply_ref(pos_pred, delta, lambda, idx, keys, dense_table(cellStart, cellEnd), D(dp), N, s));
}

int pbf_launch_delta_apply_compact(float4* pos_pred, float4* delta, const float* lambda, const uint32_t* idx,
                                   const uint32_t* keys, const uint32_t* uk, const uint32_t* off,
                                   const uint32_t* cnt, const pbf_device_params* dp, uint32_t N, cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!pos_pred || !delta || !lambda || !idx || !keys || !uk || !off || !cnt || !valid_dp(dp))
        return PBF_ERR_INVALID;
    return from_cuda(
        pbf::launch_delta_apply_ref(pos_pred, delta, lambda, idx, keys, compact_table(uk, off, cnt), D(dp), N, s));
}

int pbf_launch_xsph(float4* vel_out, const float4* vel_in, const float4* pos_pred, const uint32_t* idx,
                    const uint32_t* keys, const uint32_t* cellStart, const uint32_t* cellEnd,
                    const pbf_device_params* dp, uint32_t N, cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!vel_out || !vel_in || !pos_pred || !idx || !keys || !cellStart || !cellEnd || !valid_dp(dp))
        return PBF_ERR_INVALID;
    if (vel_out == vel_in) return PBF_ERR_INVALID;
    return from_cuda(
        pbf::launch_xsph_ref(vel_out, vel_in, pos_pred, idx, keys, dense_table(cellStart, cellEnd), D(dp), N, s));
}

int pbf_launch_xsph_compact(float4* vel_out, const float4* vel_in, const float4* pos_pred, const uint32_t* idx,
                            const uint32_t* keys, const uint32_t* uk, const uint32_t* off, const uint32_t* cnt,
                            const pbf_device_params* dp, uint32_t N, cudaStream_t s) {
    if (N == 0) return PBF_OK;
    if (!vel_out || !vel_in || !pos_pred || !idx || !keys || !uk || !off || !cnt || !valid_dp(dp))
        return PBF_ERR_INVALID;
    if (vel_out == vel_in) return PBF_ERR_INVALID;
    return from_cuda(
        pbf::launch_xsph_ref(vel_out, vel_in, pos_pred, idx, keys, compact_table(uk, off, cnt), D(dp), N, s));
}

// ----------------------------------------------------------- handle API
int pbf_create(const pbf_sim_params* p, int grid_mode, pbf_sim** out) {
    if (!p || !out) return PBF_ERR_INVALID;
    *out = nullptr;
    if (grid_mode != PBF_GRID_DENSE && grid_mode != PBF_GRID_HASHED) return PBF_ERR_INVALID;
    if (p->solverIters < 0 || !(p->grid.cellSize > 0.f)) return PBF_ERR_INVALID;
    pbf_sim* h = new (std::nothrow) pbf_sim;
    if (!h) return PBF_ERR_OOM;
    if (!h->sim.initialize(S(p), grid_mode == PBF_GRID_HASHED)) {
        cudaError_t e = cudaGetLastError();
        delete h;
        return e == cudaErrorMemoryAllocation ? PBF_ERR_OOM : (e == cudaSuccess ? PBF_ERR_INVALID : PBF_ERR_CUDA);
    }
    *out = h;
    return PBF_OK;
}

int pbf_destroy(pbf_sim* h) {
    delete h;
    return PBF_OK;
}

void* pbf_stream(pbf_sim* h) { return h ? static_cast<void*>(h->sim.cudaStream()) : nullptr; }

int pbf_set_stream(pbf_sim* h, void* stream) {
    if (!h) return PBF_ERR_INVALID;
    return h->sim.setStream(static_cast<cudaStream_t>(stream)) ? PBF_OK : PBF_ERR_CUDA;
}

int pbf_device_state(pbf_sim* h, float4** d_pos, float4** d_vel) {
    if (!h) return PBF_ERR_INVALID;
    if (d_pos) *d_pos = h->sim.devicePositionsMutable();
    if (d_vel) *d_vel = h->sim.deviceVelMutable();
    return PBF_OK;
}

int pbf_upload_state(pbf_sim* h, const float4* hp, const float4* hv) {
    if (!h || !hp || !hv) return PBF_ERR_INVALID;
    const size_t bytes = sizeof(float4) * h->sim.activeParticleCount();
    cudaStream_t s = h->sim.cudaStream();
    cudaMemcpyAsync(h->sim.devicePositionsMutable(), hp, bytes, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(h->sim.deviceVelMutable(), hv, bytes, cudaMemcpyHostToDevice, s);
    return from_cuda(cudaStreamSynchronize(s));
}

int pbf_download_state(pbf_sim* h, float4* hp, float4* hv) {
    if (!h) return PBF_ERR_INVALID;
    const size_t bytes = sizeof(float4) * h->sim.activeParticleCount();
    cudaStream_t s = h->sim.cudaStream();
    if (hp) cudaMemcpyAsync(hp, h->sim.devicePositions(), bytes, cudaMemcpyDeviceToHost, s);
    if (hv) cudaMemcpyAsync(hv, h->sim.deviceVel(), bytes, cudaMemcpyDeviceToHost, s);
    return from_cuda(cudaStreamSynchronize(s));
}

int pbf_step(pbf_sim* h, const pbf_sim_params* p) {
    if (!h) return PBF_ERR_INVALID;
    const sim::SimParams& sp = p ? S(p) : h->sim.params();
    if (sp.solverIters < 0 || !(sp.grid.cellSize > 0.f)) return PBF_ERR_INVALID;
    if (!h->sim.step(sp)) {
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? PBF_ERR_INVALID : from_cuda(e);
    }
    return PBF_OK;
}

int pbf_step_n(pbf_sim* h, const pbf_sim_params* p, int n) {
    for (int i = 0; i < n; ++i) {
        int st = pbf_step(h, p);
        if (st != PBF_OK) return st;
    }
    return PBF_OK;
}

int pbf_step_host(pbf_sim* h, const pbf_sim_params* p, float4* hp, float4* hv) {
    if (!h || !hp || !hv) return PBF_ERR_INVALID;
    const size_t bytes = sizeof(float4) * h->sim.activeParticleCount();
    cudaStream_t s = h->sim.cudaStream();
    // a failed enqueue is reported as itself, before anything else is queued
    cudaError_t e = cudaMemcpyAsync(h->sim.devicePositionsMutable(), hp, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->sim.deviceVelMutable(), hv, bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return from_cuda(e);
    int st = pbf_step(h, p);
    if (st != PBF_OK) return st;
    const size_t out = sizeof(float4) * h->sim.activeParticleCount();
    e = cudaMemcpyAsync(hp, h->sim.devicePositions(), out, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hv, h->sim.deviceVel(), out, cudaMemcpyDeviceToHost, s);
    const cudaError_t se = cudaStreamSynchronize(s);
    return from_cuda(e != cudaSuccess ? e : se);
}

int pbf_profile_step(pbf_sim* h, const pbf_sim_params* p, float* ms, const char** names, int cap, int* count) {
    if (!h || !ms || cap <= 0) return PBF_ERR_INVALID;
    const sim::SimParams& sp = p ? S(p) : h->sim.params();
    const int n = h->sim.profileStep(sp, ms, names, cap);
    if (n < 0) return PBF_ERR_INVALID;
    if (count) *count = n;
    return launch_status();
}

int pbf_launches_per_step(pbf_sim* h) { return h ? h->sim.launchesPerStep() : 0; }

int pbf_set_math_mode(pbf_sim* h, int mode) {
    if (!h || (mode != PBF_MATH_EXACT && mode != PBF_MATH_FAST)) return PBF_ERR_INVALID;
    return h->sim.setMathMode(mode) ? PBF_OK : PBF_ERR_INVALID;
}

int pbf_get_math_mode(pbf_sim* h, int* mode) {
    if (!h || !mode) return PBF_ERR_INVALID;
    *mode = h->sim.mathMode();
    return PBF_OK;
}

int pbf_set_neighbour_list_capacity(pbf_sim* h, uint32_t entries) {
    if (!h) return PBF_ERR_INVALID;
    if (entries > (1u << 20)) return PBF_ERR_INVALID;
    if (!h->sim.setNeighbourListCapacity(entries)) return PBF_ERR_OOM;
    return PBF_OK;
}

int pbf_tile_shape_count(void) { return pbf::fused_tile_shape_count(); }

int pbf_tile_shape_info(int id, int* tile, int* stage_slots) {
    int t = 0, st = 0;
    if (!pbf::fused_tile_shape_info(id, t, st)) return PBF_ERR_INVALID;
    if (tile) *tile = t;
    if (stage_slots) *stage_slots = st;
    return PBF_OK;
}

int pbf_set_tile_shape(pbf_sim* h, int id) {
    if (!h || !h->sim.setTileShape(id)) return PBF_ERR_INVALID;
    return PBF_OK;
}

int pbf_get_tile_shape(pbf_sim* h, int* id) {
    if (!h || !id) return PBF_ERR_INVALID;
    *id = h->sim.tileShape();
    return PBF_OK;
}

int pbf_autotune_tile_shape(pbf_sim* h, const pbf_sim_params* p, int steps, float* ms, int* chosen) {
    if (!h || steps < 1) return PBF_ERR_INVALID;
    const sim::SimParams& sp = p ? S(p) : h->sim.params();
    if (sp.solverIters < 0 || !(sp.grid.cellSize > 0.f)) return PBF_ERR_INVALID;
    if (!h->sim.autotuneTileShape(sp, steps, ms)) {
        const cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? PBF_ERR_INVALID : from_cuda(e);
    }
    if (chosen) *chosen = h->sim.tileShape();
    return PBF_OK;
}

int pbf_neighbour_list_stats(pbf_sim* h, uint32_t* capacity, uint32_t* longest, uint32_t* overflowed, int reset) {
    if (!h) return PBF_ERR_INVALID;
    uint32_t l = 0, o = 0;
    if (!h->sim.neighbourListStats(l, o, reset != 0)) return PBF_ERR_CUDA;
    if (capacity) *capacity = h->sim.neighbourListCapacity();
    if (longest) *longest = l;
    if (overflowed) *overflowed = o;
    return PBF_OK;
}

int pbf_synchronize(pbf_sim* h) {
    if (!h) return PBF_ERR_INVALID;
    cudaError_t e = cudaStreamSynchronize(h->sim.cudaStream());
    if (e != cudaSuccess) return from_cuda(e);
    const uint32_t err = h->sim.takeDeviceError();
    if (err & pbf::kErrTimeoutBits) return PBF_ERR_TIMEOUT;
    if (err & pbf::kErrNonFiniteBit) return PBF_ERR_NONFINITE;
    if (err) return PBF_ERR_CUDA;
    return PBF_OK;
}

int pbf_density_stats(pbf_sim* h, double out[4]) {
    if (!h || !out) return PBF_ERR_INVALID;
    sim::DeviceBuffers& b = h->sim.buffers();
    sim::GridBuffers& g = h->sim.gridBuffers();
    pbf::FusedBufs f{};
    f.pos = b.d_pos;
    f.keys = g.d_cellKeys;
    f.key_s = g.d_cellKeys_sorted;
    f.perm = g.d_indices_sorted;
    f.pred_b = b.d_pred_alt;
    f.lb = g.d_cellLowerBound;
    f.sort_temp = g.d_sortTemp;
    f.sort_bytes = g.sortTempBytes;
    f.dp = b.d_params;
    f.err = b.d_err;
    f.stats_out = b.d_stats;
    f.stats_partials = b.d_stats + 4;
    pbf::FusedShape sh{};
    sh.N = h->sim.activeParticleCount();
    sh.numCells = g.numCells;
    sh.key_bits = g.keyBits;
    cudaStream_t s = h->sim.cudaStream();
    cudaError_t e = pbf::fused_density_stats(f, sh, s);
    if (e != cudaSuccess) return from_cuda(e);
    e = cudaMemcpyAsync(out, b.d_stats, 4 * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return from_cuda(e);
    return from_cuda(cudaStreamSynchronize(s));
}

int pbf_debug_fetch(pbf_sim* h, int item, void* dst, size_t bytes) {
    if (!h || !dst) return PBF_ERR_INVALID;
    sim::DeviceBuffers& b = h->sim.buffers();
    sim::GridBuffers& g = h->sim.gridBuffers();
    const uint32_t N = h->sim.activeParticleCount();
    cudaStream_t s = h->sim.cudaStream();
    const void* src = nullptr;
    size_t need = 0;
    uint32_t scalar = 0;
    switch (item) {
        case PBF_DBG_KEYS_SORTED: src = g.d_cellKeys_sorted; need = 4u * size_t(N); break;
        case PBF_DBG_PERM: src = g.d_indices_sorted; need = 4u * size_t(N); break;
        case PBF_DBG_CELL_START:
        case PBF_DBG_CELL_END: {
            if (!g.ensureRangesMaterialised()) return PBF_ERR_OOM;
            cudaError_t e = pbf::launch_lb_to_ranges(g.d_cellStart, g.d_cellEnd, g.d_cellLowerBound, g.numCells, s);
            if (e != cudaSuccess) return from_cuda(e);
            src = item == PBF_DBG_CELL_START ? g.d_cellStart : g.d_cellEnd;
            need = 4u * size_t(g.numCells);
            break;
        }
        case PBF_DBG_UNIQUE_KEYS: src = g.d_cellUniqueKeys; need = 4u * size_t(N); break;
        case PBF_DBG_OFFSETS: src = g.d_cellOffsets; need = 4u * (size_t(N) + 1); break;
        case PBF_DBG_COMPACT_COUNT: src = g.d_compactCount; need = 4u; break;
        case PBF_DBG_LAMBDA: {
            pbf::FusedBufs f{};
            f.lam_s = b.d_lambda;
            f.perm = g.d_indices_sorted;
            pbf::FusedShape sh{};
            sh.N = N;
            cudaError_t e = pbf::fused_scatter_lambda(f, sh, b.d_lambda_by_id, s);
            if (e != cudaSuccess) return from_cuda(e);
            src = b.d_lambda_by_id;
            need = 4u * size_t(N);
            break;
        }
        case PBF_DBG_NUM_CELLS: scalar = g.numCells; need = 4u; break;
        default: return PBF_ERR_INVALID;
    }
    if (bytes != need) return PBF_ERR_INVALID;
    if (item == PBF_DBG_NUM_CELLS) {
        std::memcpy(dst, &scalar, 4);
        return PBF_OK;
    }
    cudaError_t e = cudaMemcpyAsync(dst, src, need, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return from_cuda(e);
    return from_cuda(cudaStreamSynchronize(s));
}

int pbf_debug_eval_math(int fn, const float* a, const float* b, float* out, uint32_t n) {
    if (n == 0) return PBF_OK;
    if (!a || !out || (fn != 1 && fn != 3 && !b) || fn < 0 || fn > 3) return PBF_ERR_INVALID;
    cudaError_t e = pbf::eval_math(fn, a, b, out, n, 0);
    if (e != cudaSuccess) return from_cuda(e);
    return from_cuda(cudaDeviceSynchronize());
}

int pbf_selftest_powf4(uint64_t* mismatches, uint32_t* first_mismatch_bits) {
    if (!mismatches) return PBF_ERR_INVALID;
    unsigned long long* dm = nullptr;
    uint32_t* df = nullptr;
    if (cudaMalloc(&dm, sizeof(*dm)) != cudaSuccess || cudaMalloc(&df, sizeof(*df)) != cudaSuccess) {
        cudaFree(dm);
        return PBF_ERR_OOM;
    }
    // n passes through a volatile host variable so the kernel sees it only at run time
    volatile float four = 4.0f;
    cudaError_t e = pbf::selftest_powf4(four, dm, df, 0);
    unsigned long long hm = 0;
    uint32_t hf = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&hm, dm, sizeof(hm), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&hf, df, sizeof(hf), cudaMemcpyDeviceToHost);
    cudaFree(dm);
    cudaFree(df);
    if (e != cudaSuccess) return from_cuda(e);
    *mismatches = hm;
    if (first_mismatch_bits) *first_mismatch_bits = hf;
    return PBF_OK;
}

int pbf_selftest_bounded_wait(uint32_t spin_limit, void* d_scratch) {
    if (!d_scratch) return PBF_ERR_INVALID;
    uint32_t* w = static_cast<uint32_t*>(d_scratch);
    cudaError_t e = pbf::selftest_bounded_wait(spin_limit, w, 0);
    if (e != cudaSuccess) return from_cuda(e);
    uint32_t host[4] = {0, 0, 0, 0};
    e = cudaMemcpy(host, w, sizeof(host), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return from_cuda(e);
    return (host[1] & pbf::kErrLookbackTimeoutBit) ? PBF_ERR_TIMEOUT : PBF_OK;
}

int pbf_selftest_stage_wait(uint32_t spin_limit, void* d_scratch) {
    if (!d_scratch) return PBF_ERR_INVALID;
    uint32_t* w = static_cast<uint32_t*>(d_scratch);
    cudaError_t e = pbf::fused_selftest_stage_wait(spin_limit, w, 0);
    if (e != cudaSuccess) return from_cuda(e);
    uint32_t host = 0;
    e = cudaMemcpy(&host, w, sizeof(host), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return from_cuda(e);
    return (host & pbf::kErrStageTimeoutBit) ? PBF_ERR_TIMEOUT : PBF_OK;
}

// ------------------------------------------- reference-name entry points
// Exact symbols and signatures of the reference's extern "C" launchers, so a
// reference build can link this library instead of compiling sim/*.cu.

void LaunchIntegratePred(float4* posCurr, const float4* velSrc, float4* posPred, float3 gravity, float dt,
                         uint32_t N, cudaStream_t s) {
    if (!posCurr || !velSrc || !posPred || N == 0) return;
    pbf::launch_integrate_pred_ref(posCurr, velSrc, posPred, gravity, dt, N, s);
}

void LaunchBoundary(float4* pos_pred, float4* vel, sim::GridBounds grid, float restitution, uint32_t N,
                    cudaStream_t s) {
    pbf::launch_boundary_ref(pos_pred, vel, grid, restitution, N, s);
}

void LaunchVelocity(float4* vel, const float4* pos, const float4* pos_pred, float inv_dt, uint32_t N,
                    cudaStream_t s) {
    pbf::launch_velocity_ref(vel, pos, pos_pred, inv_dt, N, s);
}

void LaunchHashKeys(uint32_t* keys, uint32_t* indices, const float4* pos, sim::GridBounds grid, uint32_t N,
                    cudaStream_t s) {
    pbf::launch_hash_keys_ref(keys, indices, pos, grid, N, s);
}

void LaunchSortPairsQuery(size_t* tempBytes, const uint32_t*, uint32_t*, const uint32_t*, uint32_t*, uint32_t N,
                          cudaStream_t) {
    if (tempBytes) *tempBytes = pbf::sort_temp_bytes(N, 32);
}

void LaunchSortPairs(void* d_temp_storage, size_t tempBytes, uint32_t* d_keys_in, uint32_t* d_keys_out,
                     uint32_t* d_vals_in, uint32_t* d_vals_out, uint32_t N, cudaStream_t s) {
    pbf::sort_pairs(d_temp_storage, tempBytes, d_keys_in, d_keys_out, d_vals_in, d_vals_out, N, 32, s, nullptr);
}

void LaunchCellRanges(uint32_t* cellStart, uint32_t* cellEnd, const uint32_t* keysSorted, uint32_t N,
                      uint32_t numCells, cudaStream_t s) {
    pbf::launch_cell_ranges_ref(cellStart, cellEnd, keysSorted, N, numCells, s);
}

bool EnsureCellCompactScratch(uint32_t N, uint32_t) { return ensure_global_compact_scratch(N); }

void LaunchCellRangesCompact(uint32_t* d_uniqueKeys, uint32_t* d_offsets, uint32_t* d_compactCount,
                             const uint32_t* d_keysSorted, uint32_t N, cudaStream_t s) {
    if (N > 0 && !ensure_global_compact_scratch(N)) return;
    pbf::launch_compact(g_compactScratch, g_compactScratchBytes, d_uniqueKeys, d_offsets, d_compactCount, nullptr,
                        d_keysSorted, N, s, nullptr);
}

void LaunchLambda(float* lambda, const float4* pos_pred, const uint32_t* idx, const uint32_t* keys,
                  const uint32_t* cellStart, const uint32_t* cellEnd, sim::DeviceParams dp, uint32_t N,
                  cudaStream_t s) {
    pbf::launch_lambda_ref(lambda, pos_pred, idx, keys, dense_table(cellStart, cellEnd), dp, N, s);
}

void LaunchLambdaCompact(float* lambda, const float4* pos_pred, const uint32_t* idx, const uint32_t* keys,
                         const uint32_t* uk, const uint32_t* off, const uint32_t* cnt, sim::DeviceParams dp,
                         uint32_t N, cudaStream_t s) {
    pbf::launch_lambda_ref(lambda, pos_pred, idx, keys, compact_table(uk, off, cnt), dp, N, s);
}

void LaunchDeltaApply(float4* pos_pred, float4* delta, const float* lambda, const uint32_t* idx,
                      const uint32_t* keys, const uint32_t* cellStart, const uint32_t* cellEnd,
                      sim::DeviceParams dp, uint32_t N, cudaStream_t s) {
    pbf::launch_delta_apply_ref(pos_pred, delta, lambda, idx, keys, dense_table(cellStart, cellEnd), dp, N, s);
}

void LaunchDeltaApplyCompact(float4* pos_pred, float4* delta, const float* lambda, const uint32_t* idx,
                             const uint32_t* keys, const uint32_t* uk, const uint32_t* off, const uint32_t* cnt,
                             sim::DeviceParams dp, uint32_t N, cudaStream_t s) {
    pbf::launch_delta_apply_ref(pos_pred, delta, lambda, idx, keys, compact_table(uk, off, cnt), dp, N, s);
}

// The reference calls these with vel_out == vel_in (sim/post_ops.cpp:59,65).
// That in-place form is a data race; here it is made Jacobi by reading a
// stream-ordered snapshot of the old velocities.
static void xsph_ref_entry(float4* vel_out, const float4* vel_in, const float4* pos_pred, const uint32_t* idx,
                           const uint32_t* keys, const pbf::RefTable& t, const sim::DeviceParams& dp, uint32_t N,
                           cudaStream_t s) {
    if (N == 0 || !(dp.xsph_c > 0.f)) return;
    if (vel_out != vel_in) {
        pbf::launch_xsph_ref(vel_out, vel_in, pos_pred, idx, keys, t, dp, N, s);
        return;
    }
    float4* snap = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void**>(&snap), sizeof(float4) * N, s) != cudaSuccess) return;
    cudaMemcpyAsync(snap, vel_in, sizeof(float4) * N, cudaMemcpyDeviceToDevice, s);
    pbf::launch_xsph_ref(vel_out, snap, pos_pred, idx, keys, t, dp, N, s);
    cudaFreeAsync(snap, s);
}

void LaunchXSPH(float4* vel_out, const float4* vel_in, const float4* pos_pred, const uint32_t* idx,
                const uint32_t* keys, const uint32_t* cellStart, const uint32_t* cellEnd, sim::DeviceParams dp,
                uint32_t N, cudaStream_t s) {
    xsph_ref_entry(vel_out, vel_in, pos_pred, idx, keys, dense_table(cellStart, cellEnd), dp, N, s);
}

void LaunchXSPHCompact(float4* vel_out, const float4* vel_in, const float4* pos_pred, const uint32_t* idx,
                       const uint32_t* keys, const uint32_t* uk, const uint32_t* off, const uint32_t* cnt,
                       sim::DeviceParams dp, uint32_t N, cudaStream_t s) {
    xsph_ref_entry(vel_out, vel_in, pos_pred, idx, keys, compact_table(uk, off, cnt), dp, N, s);
}

}  // extern "C"
