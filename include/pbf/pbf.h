/*
 * pbf.h - C ABI of the GB300 PBF step library (libpbf_gb300.so).
 *
 * Three layers, all extern "C", plain pointers and sizes, no C++ or torch
 * types:
 *
 *  1. Phase launchers  pbf_launch_*  - one per reference launcher, same
 *     argument order and meaning as the reference's extern "C" Launch*
 *     functions (cited per entry), returning a status code instead of void.
 *     Buffers use the reference's layout: particle arrays indexed by the
 *     original particle id, neighbour tables indexed through indicesSorted.
 *     The exact reference symbol names (LaunchHashKeys, ...) are exported too,
 *     see launch_abi.h.
 *  2. Whole-step handle  pbf_create / pbf_step / ...  - the fused GB300 step
 *     (the reference's sim::Simulator::step, sim/simulator.cpp:560-643, with
 *     the commit swap of :144-159 folded in).
 *  3. Helpers: parameter construction (console::BuildSimParams semantics,
 *     engine/core/console.cpp:198-267), seeded scene generation.
 *
 * Every call returns pbf_status (0 = PBF_OK).  No call aborts or traps.
 * All device pointers are caller-owned unless stated otherwise; launchers
 * never allocate.  Stream arguments are cudaStream_t (0 = legacy default).
 */
#ifndef PBF_H
#define PBF_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime_api.h>
#include "pbf_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef enum pbf_status {
    PBF_OK = 0,
    PBF_ERR_INVALID = 1,     /* bad argument / size / aliasing */
    PBF_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    PBF_ERR_OOM = 3,         /* device or host allocation failed */
    PBF_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    PBF_ERR_NONFINITE = 5,   /* NaN/Inf detected in particle state */
    PBF_ERR_UNSUPPORTED = 6  /* feature/size outside what this build handles */
} pbf_status;

const char* pbf_status_string(int status);
int pbf_version(void); /* major*10000 + minor*100 + patch */
/* sizeof of pbf_kernel_coeffs, pbf_grid_bounds, pbf_tuning, pbf_sim_params,
 * pbf_device_params as compiled into the library (ABI check for bindings). */
void pbf_abi_sizes(uint32_t out[5]);

/* -------------------------------------------------------------- parameters */
/* Defaults of sim::PbfTuning (reference sim/parameters.h:27-57). */
void pbf_default_tuning(pbf_tuning* out);
/* sim::MakeKernelCoeffs (sim/parameters.h:94-107). */
void pbf_make_kernel_coeffs(float h, pbf_kernel_coeffs* out);
/* sim::MakeDeviceParams (sim/parameters.h:109-123). */
void pbf_make_device_params(const pbf_sim_params* sp, pbf_device_params* out);
/* GridSystem::ComputeDims (sim/grid_system.h:9-17): ceil(extent/cellSize). */
void pbf_compute_dims(const pbf_grid_bounds* g, int32_t out_dim[3]);

/* Dam-break scene constants used by every plain-path configuration:
 * particle radius r = 0.005, lattice spacing 0.01 = 2r, h = 2.5f*r,
 * cell = h, rest density from the unjittered lattice (self term excluded,
 * sim/pbf_lambda.cu:63), mass = 1000 * spacing^3, dt = 1/120, gravity
 * (0,-9.8,0), lambda_denom_eps = 100, s_corr k=0.1 n=4 dq=0.2h, XSPH c=0.01,
 * XPBD off, maxNeighbors 64, restitution 0; box [0, box_max].
 * num_particles is stored in numParticles/maxParticles. */
int pbf_dam_break_params(float box_max_x, float box_max_y, float box_max_z,
                         int solver_iters, uint32_t num_particles,
                         pbf_sim_params* out);

/* Seeded lattice of nx*ny*nz particles at origin + (ix,iy,iz)*spacing with a
 * per-axis uniform jitter in [-jitter, +jitter] drawn from
 * std::mt19937_64(seed) (3 draws per particle, x,y,z), clamped into
 * [box_min, box_max]; w = 1.  Particle order: x fastest, then y, then z
 * (as sim::Simulator::seedBoxLattice, sim/simulator.cpp:831-846).
 * pos_out must hold nx*ny*nz float4 (host memory). */
int pbf_seed_lattice(float4* pos_out, uint32_t nx, uint32_t ny, uint32_t nz,
                     float origin_x, float origin_y, float origin_z,
                     float spacing, float jitter, uint64_t seed,
                     const pbf_grid_bounds* clamp_box);

/* ------------------------------------------------------- phase launchers */
/* sim/integrate.cu:76-89 LaunchIntegratePred: posPred = pos + (vel + g dt) dt,
 * posPred.w = pos.w. */
int pbf_launch_integrate_pred(const float4* posCurr, const float4* velSrc,
                              float4* posPred, float3 gravity, float dt,
                              uint32_t N, cudaStream_t s);
/* sim/boundary.cu:37-40 LaunchBoundary: clamp into the AABB, reflect the
 * offending velocity component by -restitution, pos.w = 1, vel.w = 0. */
int pbf_launch_boundary(float4* pos_pred, float4* vel, const pbf_grid_bounds* grid,
                        float restitution, uint32_t N, cudaStream_t s);
/* sim/boundary.cu:41-44 LaunchVelocity: vel = (pos_pred - pos) * inv_dt, w = 0. */
int pbf_launch_velocity(float4* vel, const float4* pos, const float4* pos_pred,
                        float inv_dt, uint32_t N, cudaStream_t s);
/* sim/hash_keys.cu:30-34 LaunchHashKeys: keys[i] = clamped linear cell of
 * pos[i], indices[i] = i. */
int pbf_launch_hash_keys(uint32_t* keys, uint32_t* indices, const float4* pos,
                         const pbf_grid_bounds* grid, uint32_t N, cudaStream_t s);

/* sim/sort_pairs.cu:5-16 LaunchSortPairsQuery: temp bytes for N pairs. */
int pbf_sort_pairs_query(size_t* tempBytes, uint32_t N);
/* sim/sort_pairs.cu:18-27 LaunchSortPairs: stable ascending sort of
 * (keys_in, vals_in) over key bits [0,32) into (keys_out, vals_out), by a
 * onesweep LSD radix sort (8-bit digits, decoupled look-back).  Passes whose
 * digit is the same for every key are skipped.  The inputs are left intact. */
int pbf_launch_sort_pairs(void* d_temp, size_t tempBytes,
                          const uint32_t* keys_in, uint32_t* keys_out,
                          const uint32_t* vals_in, uint32_t* vals_out,
                          uint32_t N, cudaStream_t s);
/* Same sort restricted to key bits [0, num_bits). */
int pbf_launch_sort_pairs_bits(void* d_temp, size_t tempBytes,
                               const uint32_t* keys_in, uint32_t* keys_out,
                               const uint32_t* vals_in, uint32_t* vals_out,
                               uint32_t N, int num_bits, cudaStream_t s);

/* sim/cell_ranges.cu:55-80 LaunchCellRanges: dense per-cell [start, end);
 * empty cells get start = 0xFFFFFFFF, end = 0.  Writes every cell (no
 * separate memsets needed). */
int pbf_launch_cell_ranges(uint32_t* cellStart, uint32_t* cellEnd,
                           const uint32_t* keysSorted, uint32_t N,
                           uint32_t numCells, cudaStream_t s);

/* Scratch for pbf_launch_cell_ranges_compact (replaces the reference's
 * process-global scratch of sim/cell_compact.cu:50-93). */
int pbf_cell_compact_scratch_query(size_t* bytes, uint32_t N);
/* sim/cell_compact.cu:187-231 LaunchCellRangesCompact: uniqueKeys[m],
 * offsets[m] = first sorted position of segment m, offsets[M] = N,
 * *compactCount = M.  Segment starts are found with __match_any_sync and
 * placed with a single-pass decoupled look-back scan.  Its waits are
 * bounded: if one gives up (a GPU that starved a predecessor tile for over
 * 2^22 polls), *compactCount is set to 0xFFFFFFFF and the table is invalid;
 * this library's compact-table launchers clamp such a count to N, so they
 * stay in bounds. */
int pbf_launch_cell_ranges_compact(void* d_scratch, size_t scratchBytes,
                                   uint32_t* uniqueKeys, uint32_t* offsets,
                                   uint32_t* compactCount,
                                   const uint32_t* keysSorted, uint32_t N,
                                   cudaStream_t s);

/* No counterpart in the reference.  The same compaction as
 * pbf_launch_cell_ranges_compact, for callers that cannot allocate device
 * memory while they run (a frame loop where cudaMalloc/cudaFree would
 * synchronize the device, a plugin host that hands out no GPU memory): its
 * scratch is one fixed device array inside the library, so the caller passes
 * only inputs and outputs.  At most 16,777,216 keys per call (larger N:
 * PBF_ERR_UNSUPPORTED, nothing launched).  The first call on a device looks
 * up the array's device address (once per device, with that device current);
 * make that first call before any stream capture; the address is looked up
 * again when the current device's context changes (e.g. after
 * cudaDeviceReset).  All calls share the array: each clears what must start
 * at zero, but calls that overlap on the GPU race - serialize them.  A
 * look-back that gives up is reported as in pbf_launch_cell_ranges_compact
 * (*compactCount = 0xFFFFFFFF). */
int pbf_launch_cell_ranges_compact_noalloc(uint32_t* uniqueKeys, uint32_t* offsets,
                                           uint32_t* compactCount,
                                           const uint32_t* keysSorted, uint32_t N,
                                           cudaStream_t s);

/* sim/pbf_lambda.cu:246-258 LaunchLambda (dense table).  lambda[i] for every
 * particle i; the reference writes through device globals bound to the same
 * buffers, this entry point uses its arguments. */
int pbf_launch_lambda(float* lambda, const float4* pos_pred,
                      const uint32_t* indicesSorted, const uint32_t* keysSorted,
                      const uint32_t* cellStart, const uint32_t* cellEnd,
                      const pbf_device_params* dp, uint32_t N, cudaStream_t s);
/* sim/pbf_lambda.cu:260-274 LaunchLambdaCompact (compact table). */
int pbf_launch_lambda_compact(float* lambda, const float4* pos_pred,
                              const uint32_t* indicesSorted, const uint32_t* keysSorted,
                              const uint32_t* uniqueKeys, const uint32_t* offsets,
                              const uint32_t* compactCount,
                              const pbf_device_params* dp, uint32_t N, cudaStream_t s);
/* sim/pbf_delta_apply.cu:239-258 LaunchDeltaApply: delta[i] then pos_pred += delta. */
int pbf_launch_delta_apply(float4* pos_pred, float4* delta, const float* lambda,
                           const uint32_t* indicesSorted, const uint32_t* keysSorted,
                           const uint32_t* cellStart, const uint32_t* cellEnd,
                           const pbf_device_params* dp, uint32_t N, cudaStream_t s);
/* sim/pbf_delta_apply.cu:260-280 LaunchDeltaApplyCompact. */
int pbf_launch_delta_apply_compact(float4* pos_pred, float4* delta, const float* lambda,
                                   const uint32_t* indicesSorted, const uint32_t* keysSorted,
                                   const uint32_t* uniqueKeys, const uint32_t* offsets,
                                   const uint32_t* compactCount,
                                   const pbf_device_params* dp, uint32_t N, cudaStream_t s);
/* sim/xsph.cu:189-205 LaunchXSPH, Jacobi form: vel_out must not alias vel_in
 * (PBF_ERR_INVALID otherwise).  No-op when dp->xsph_c <= 0. */
int pbf_launch_xsph(float4* vel_out, const float4* vel_in, const float4* pos_pred,
                    const uint32_t* indicesSorted, const uint32_t* keysSorted,
                    const uint32_t* cellStart, const uint32_t* cellEnd,
                    const pbf_device_params* dp, uint32_t N, cudaStream_t s);
/* sim/xsph.cu:207-228 LaunchXSPHCompact, Jacobi form. */
int pbf_launch_xsph_compact(float4* vel_out, const float4* vel_in, const float4* pos_pred,
                            const uint32_t* indicesSorted, const uint32_t* keysSorted,
                            const uint32_t* uniqueKeys, const uint32_t* offsets,
                            const uint32_t* compactCount,
                            const pbf_device_params* dp, uint32_t N, cudaStream_t s);

/* ------------------------------------------------------ whole-step handle */
typedef struct pbf_sim pbf_sim;

/* Grid strategy: PBF_GRID_DENSE = per-cell start/end table
 * (sim/phases.cpp:56-60), PBF_GRID_HASHED = compact unique-key table
 * (console perf.use_hashed_grid, sim/phases.cpp:54). */
enum { PBF_GRID_DENSE = 0, PBF_GRID_HASHED = 1 };

/* sim::Simulator::initialize (sim/simulator.cpp:217-296): allocates every
 * buffer for max(numParticles, maxParticles) particles and the grid of
 * p->grid (dims recomputed with ComputeDims).  Owns a non-blocking stream. */
int pbf_create(const pbf_sim_params* p, int grid_mode, pbf_sim** out);
int pbf_destroy(pbf_sim* sim);
/* The stream the handle enqueues its work on (cudaStream_t): its own
 * non-blocking stream unless pbf_set_stream chose another. */
void* pbf_stream(pbf_sim* sim);
/* Enqueue the handle's work (steps, copies, profiling) on a caller's stream
 * from now on, as the reference's launchers take one (sim/phases.cpp:8-25);
 * NULL returns to the handle's own stream.  The switch waits for the work
 * already queued on the previous stream.  The step graph is still captured
 * on the handle's own stream and launched on the chosen one. */
int pbf_set_stream(pbf_sim* sim, void* stream);
/* Device pointers of the committed state (float4[N], original particle order). */
int pbf_device_state(pbf_sim* sim, float4** d_pos, float4** d_vel);

/* Host <-> device state copies (blocking).  N = numParticles of the handle. */
int pbf_upload_state(pbf_sim* sim, const float4* h_pos, const float4* h_vel);
int pbf_download_state(pbf_sim* sim, float4* h_pos, float4* h_vel);

/* One simulation step (sim::Simulator::step): launch the captured step graph
 * on the handle's stream, asynchronously.  p may be NULL (parameters
 * unchanged); a structural change (numParticles, solverIters, maxNeighbors,
 * grid) re-captures the graph, any other change is uploaded to the
 * device-resident parameter block before the launch. */
int pbf_step(pbf_sim* sim, const pbf_sim_params* p);
/* n steps back to back (same parameters). */
int pbf_step_n(pbf_sim* sim, const pbf_sim_params* p, int n);
/* End-to-end step on HOST buffers: copy h_pos/h_vel to the device, one step,
 * copy the new state back, synchronize.  h_pos/h_vel should be pinned. */
int pbf_step_host(pbf_sim* sim, const pbf_sim_params* p, float4* h_pos, float4* h_vel);
/* One step launched phase by phase (not as a graph) with CUDA events between
 * the launches, on the handle's stream; advances the state like pbf_step.
 * Writes up to cap entries: ms[k] = device time of phase k, names[k] = its
 * name (static strings); *count = number of phases (predict_keys, sort,
 * gather_tables, lambda_1, delta_1, ..., commit). */
int pbf_profile_step(pbf_sim* sim, const pbf_sim_params* p, float* ms, const char** names, int cap, int* count);
/* Kernel launches of this library in one pbf_step (graph nodes that are
 * kernels of libpbf_gb300; memsets excluded). */
int pbf_launches_per_step(pbf_sim* sim);
/* Wait for the stream and report any device-side error flag:
 * PBF_ERR_TIMEOUT when a bounded wait gave up, PBF_ERR_NONFINITE when a step
 * committed a NaN or Inf position or velocity (the state is kept as
 * computed).  The flags clear once reported. */
int pbf_synchronize(pbf_sim* sim);

/* Neighbour lists.  No counterpart in the reference, whose solver passes
 * each walk the whole 27-cell stencil.  Here the candidates within
 * h + 2 * (position updates covered) * disp_clamp_max_h * h of each particle are
 * listed once per step (once per span of solver iterations), in the stencil's
 * order, and the lambda, delta and XSPH passes walk those lists; results are
 * identical.  Lists are used only while the displacement clamp is on.
 * entries = capacity per particle, rounded up to a multiple of 8 (default
 * 512; 4 bytes of device memory per entry and particle); a particle with a
 * longer list makes its warp walk the stencil.  0 turns lists off.  Takes
 * effect at the next step. */
int pbf_set_neighbour_list_capacity(pbf_sim* sim, uint32_t entries);
/* *capacity = current capacity (0 = off); *longest = longest list built and
 * *overflowed = lists longer than the capacity, both since the last reset
 * (reset != 0 clears them after reading).  Any output may be NULL. */
int pbf_neighbour_list_stats(pbf_sim* sim, uint32_t* capacity, uint32_t* longest, uint32_t* overflowed, int reset);

/* Tile shapes of the neighbour passes (no counterpart in the reference): a
 * CTA takes `tile` consecutive sorted particles and stages up to
 * `stage_slots` neighbour slots in shared memory.  Every shape computes the
 * same results; which is fastest depends on the scene.  Shapes are numbered
 * 0 .. pbf_tile_shape_count() - 1 (0 is the default). */
int pbf_tile_shape_count(void);
int pbf_tile_shape_info(int id, int* tile, int* stage_slots);
/* Selects the shape for the following steps (PBF_ERR_INVALID for an unknown id). */
int pbf_set_tile_shape(pbf_sim* sim, int id);
int pbf_get_tile_shape(pbf_sim* sim, int* id);
/* Autotuner: times `steps` steps of every shape from the current state (one
 * untimed step per shape first), then restores the state, clears the list
 * statistics and selects the fastest shape.  ms (pbf_tile_shape_count()
 * floats, may be NULL) receives each shape's mean step time; *chosen (may be
 * NULL) the selected shape.  Synchronous. */
int pbf_autotune_tile_shape(pbf_sim* sim, const pbf_sim_params* p, int steps, float* ms, int* chosen);

/* Arithmetic of the delta pass (no counterpart in the reference).
 * PBF_MATH_EXACT (the default) evaluates the reference kernels' operations
 * with their rounding: keys, permutation, cell tables, lambda, positions and
 * velocities are bit-identical to the reference's FP32 kernels.
 * PBF_MATH_FAST computes the s_corr power for the default exponent n = 4
 * from error-free products (ratio^4 correctly rounded except next to a
 * rounding tie) instead of CUDA's powf, whose results are an ulp off for
 * 6.3% of inputs.  Everything else is the exact mode's: keys, permutation,
 * cell tables and the first iteration's lambda stay bit-exact; lambda,
 * positions and velocities agree with the exact mode within 1e-5 relative
 * per step.  Takes effect at the next step. */
enum { PBF_MATH_EXACT = 0, PBF_MATH_FAST = 1 };
int pbf_set_math_mode(pbf_sim* sim, int mode);
int pbf_get_math_mode(pbf_sim* sim, int* mode);

/* Density-constraint diagnostics of the committed state, uncapped neighbour
 * sums over the step's cell grid: out[0] = mean |rho_i/rho0 - 1|,
 * out[1] = max |rho_i/rho0 - 1|, out[2] = mean max(rho_i/rho0 - 1, 0),
 * out[3] = mean neighbour count.  Deterministic (fixed-order reduction). */
int pbf_density_stats(pbf_sim* sim, double out[4]);

/* Test/inspection access to the last step's intermediates (blocking copy to
 * host).  See PBF_DBG_*; bytes must match the item's size. */
enum {
    PBF_DBG_KEYS_SORTED = 0,   /* uint32[N] cell key per sorted slot */
    PBF_DBG_PERM = 1,          /* uint32[N] original id per sorted slot */
    PBF_DBG_CELL_START = 2,    /* uint32[numCells] reference dense format */
    PBF_DBG_CELL_END = 3,      /* uint32[numCells] */
    PBF_DBG_UNIQUE_KEYS = 4,   /* uint32[N] (first compactCount valid; hashed) */
    PBF_DBG_OFFSETS = 5,       /* uint32[N+1] (first compactCount+1 valid) */
    PBF_DBG_COMPACT_COUNT = 6, /* uint32[1] */
    PBF_DBG_LAMBDA = 7,        /* float[N] last iteration's lambda by original id */
    PBF_DBG_NUM_CELLS = 8      /* uint32[1] */
};
int pbf_debug_fetch(pbf_sim* sim, int item, void* host_dst, size_t bytes);

/* --------------------------------------------------------- batched ensemble */
/* Many independent scenes stepped as one workload.  No counterpart in the
 * reference, which steps one scene per sim::Simulator (sim/simulator.cpp:
 * 560-643), so a batch there is a loop over simulators.  scenes[s] holds scene
 * s's parameters (numParticles, grid box and cell size, gravity, dt, kernel,
 * tuning, solverIters); the state is the scenes' particles concatenated,
 * scene s owning [offsets[s], offsets[s+1]).  Every scene evolves exactly as a
 * pbf_sim with the same parameters (bit-identical), with one launch per phase
 * over all scenes and the step captured in one CUDA graph.  Parameters are
 * fixed at creation.  PBF_ERR_UNSUPPORTED when the scenes' particles or cells
 * exceed 2^32 - 16 in total. */
typedef struct pbf_ensemble pbf_ensemble;
int pbf_ensemble_create(const pbf_sim_params* scenes, uint32_t num_scenes, pbf_ensemble** out);
int pbf_ensemble_destroy(pbf_ensemble* ens);
void* pbf_ensemble_stream(pbf_ensemble* ens);
/* As pbf_set_stream, for an ensemble. */
int pbf_ensemble_set_stream(pbf_ensemble* ens, void* stream);
uint32_t pbf_ensemble_num_particles(pbf_ensemble* ens);
/* offsets: num_scenes + 1 entries. */
int pbf_ensemble_scene_offsets(pbf_ensemble* ens, uint32_t* offsets);
int pbf_ensemble_upload_state(pbf_ensemble* ens, const float4* pos, const float4* vel);
int pbf_ensemble_download_state(pbf_ensemble* ens, float4* pos, float4* vel);
/* n steps, enqueued on the ensemble's stream (asynchronous). */
int pbf_ensemble_step(pbf_ensemble* ens, int n);
/* One step from and back to host state (pinned memory recommended). */
int pbf_ensemble_step_host(pbf_ensemble* ens, float4* pos, float4* vel);
int pbf_ensemble_synchronize(pbf_ensemble* ens);
int pbf_ensemble_launches_per_step(pbf_ensemble* ens);
/* Tile shape of the ensemble's neighbour passes (see pbf_tile_shape_count)
 * and its autotuner, as for a single simulation: every shape is timed over
 * `steps` steps from the current state, the state is restored and the
 * fastest shape kept (the step graph is re-captured for it). */
int pbf_ensemble_set_tile_shape(pbf_ensemble* ens, int id);
int pbf_ensemble_get_tile_shape(pbf_ensemble* ens, int* id);
/* Arithmetic mode of the ensemble's delta pass (see pbf_set_math_mode);
 * the step graph is captured again. */
int pbf_ensemble_set_math_mode(pbf_ensemble* ens, int mode);
int pbf_ensemble_get_math_mode(pbf_ensemble* ens, int* mode);
int pbf_ensemble_autotune(pbf_ensemble* ens, int steps, float* ms, int* chosen);

/* ----------------------------------------------------------------- adjoint */
/* Reverse-mode gradients of the step.  No counterpart in the reference.
 * pbf_forward advances the handle's scene `steps` steps (its current
 * parameters) and records (pos, vel) checkpoints every `checkpoint_every`
 * steps in a tape.  pbf_backward takes dL/d(final positions) and dL/d(final
 * velocities) (device float4[N], particle order, w ignored) and writes
 * dL/d(initial positions), dL/d(initial velocities) (device float4[N], may
 * be NULL) and dL/d(xsph_c) (host).  It replays each checkpoint segment once,
 * recording every step's intermediates, and differentiates the steps in
 * reverse, with each step's neighbour sets held fixed and clamps passing the
 * derivative of the branch taken.  Device memory: 32 bytes per particle per
 * checkpoint plus (16 (iters + 3) + 12) bytes per particle and the cell table
 * per step of a segment.  PBF_ERR_UNSUPPORTED for XPBD (xpbd_enable). */
typedef struct pbf_tape pbf_tape;
int pbf_forward(pbf_sim* sim, int steps, int checkpoint_every, pbf_tape** tape);
int pbf_backward(pbf_tape* tape, const float4* d_pos_bar, const float4* d_vel_bar, float4* d_pos0_bar,
                 float4* d_vel0_bar, float* xsph_c_bar);
int pbf_tape_destroy(pbf_tape* tape);
/* Batched adjoint over `count` independent scenes, one handle each: the
 * same tapes and gradients as pbf_forward / pbf_backward called scene by
 * scene, but every scene's steps are enqueued (each on its handle's or its
 * tape's stream) before any is waited for, so the scenes run side by side on
 * the GPU, and each call synchronises once.  The handles (and the tapes) must
 * be distinct; the tapes of one backward batch must have the same steps and
 * checkpoint interval.  Arrays are indexed by scene: tapes[count] (out, all
 * NULL on failure), d_pos_bar / d_vel_bar[count] (device pointers),
 * d_pos0_bar / d_vel0_bar[count] (the arrays or their entries may be NULL)
 * and xsph_c_bar (host float[count], may be NULL). */
int pbf_forward_batch(pbf_sim* const* sims, int count, int steps, int checkpoint_every, pbf_tape** tapes);
int pbf_backward_batch(pbf_tape* const* tapes, int count, const float4* const* d_pos_bar,
                       const float4* const* d_vel_bar, float4* const* d_pos0_bar, float4* const* d_vel0_bar,
                       float* xsph_c_bar);
/* SPH density of the handle's state on res^3 cell centres of its grid box:
 * rho(g) = sum_i m W_poly6(|g - p_i|), into device float[res^3].  Each
 * particle adds its terms with float atomics, so the last bits of rho (and
 * of the loss and gradient below) can differ from run to run. */
int pbf_density_grid(pbf_sim* sim, int res, float* d_grid);
/* loss = mean over the res^3 points of (rho(g) - target(g))^2 (target:
 * device float[res^3]); d_pos_bar (device float4[N], may be NULL) receives
 * dL/d(positions). */
int pbf_density_grid_loss(pbf_sim* sim, int res, const float* d_target, double* loss, float4* d_pos_bar);

/* Inspection: evaluates the device math the neighbour kernels use on
 * device arrays: fn 0 = powf(a, b), 1 = sqrtf(a), 2 = a / b (IEEE),
 * 3 = a^4 as the fast arithmetic mode computes it (b unused). */
int pbf_debug_eval_math(int fn, const float* d_a, const float* d_b, float* d_out, uint32_t n);

/* The delta kernels evaluate s_corr's (w / w_q)^n with the exponent written
 * as the constant 4 when n == 4, a form the compiler evaluates faster.  This
 * compares it with powf(x, n) for n = 4 known only at run time on every
 * non-negative float bit pattern (about 2.1e9 values): *mismatches must be 0
 * for the results to stay those of the reference kernels.
 * *first_mismatch_bits (may be NULL) = the smallest mismatching bit pattern,
 * 0xFFFFFFFF if none. */
int pbf_selftest_powf4(uint64_t* mismatches, uint32_t* first_mismatch_bits);

/* Runtime configuration (headless console::RuntimeConsole, include/pbf/console.h):
 * the reference application's defaults, CubeMix scene derivation, config.json
 * merge and RuntimeConsole -> SimParams mapping.  A console is a host object;
 * none of these calls touch the GPU except pbf_seed_cube_mix. */
typedef struct pbf_console pbf_console;
/* Defaults of the reference's RuntimeConsole, CubeMix derived (numParticles,
 * simulation box). */
int pbf_console_create(pbf_console** out);
int pbf_console_destroy(pbf_console* c);
/* Fields by name: "sim.<field>", "sim.pbf.<field>", "sim.gravity.x",
 * "sim.gridMins.y", "perf.<field>" (RuntimeConsole names).  Booleans read and
 * write 0 / 1, sim.massMode 0 (explicit), 1 (sphere by radius), 2 (uniform
 * lattice).  PBF_ERR_INVALID for an unknown name or an out-of-range value.
 * Setting CubeMix fields does not re-derive the scene: call
 * pbf_console_prepare_cube_mix. */
int pbf_console_set(pbf_console* c, const char* field, double value);
int pbf_console_get(pbf_console* c, const char* field, double* value);
int pbf_console_prepare_cube_mix(pbf_console* c);
/* Merges a config.json text ("performance", "simulation", "profile",
 * "profiles"; other sections are application state and are ignored), then
 * re-derives the CubeMix scene.  PBF_ERR_INVALID, the console unchanged and a
 * message in err (err_cap bytes, may be NULL) when the text is not JSON or a
 * known key has a value of the wrong type. */
int pbf_console_merge_json(pbf_console* c, const char* text, char* err, uint32_t err_cap);
/* Name of the active profile ("" if none); PBF_ERR_INVALID if cap is too small. */
int pbf_console_profile(pbf_console* c, char* name, uint32_t cap);
/* BuildSimParams of the reference (then, with sanitize != 0, the
 * application's clamps: solverIters [1, 64], maxNeighbors [8, neighbor cap or
 * 1024], sortEveryN >= 1), starting from a value-initialised SimParams. */
int pbf_console_build_sim_params(pbf_console* c, int sanitize, pbf_sim_params* out);
/* CubeMix group centres (x, y, z per group); xyz may be NULL to query *count. */
int pbf_console_cube_mix_centers(pbf_console* c, float* xyz, uint32_t cap, uint32_t* count);
/* Seeds the simulation's particles as the reference application does for the
 * CubeMix scene: cubes of cube_edge_particles^3 at the group centres, lattice
 * spacing h * cube_lattice_spacing_factor_h, seeded jitter.  The simulation's
 * particle count must equal the scene's. */
int pbf_seed_cube_mix(pbf_sim* sim, pbf_console* c);

/* Failure-path self-test of the bounded device waits: one block polls a
 * look-back status that nothing ever publishes.  After spin_limit polls the
 * kernel records the timeout in its error word and returns, leaving the
 * context usable.  d_scratch: caller-owned device memory of >= 16 bytes.
 * Returns PBF_ERR_TIMEOUT when the wait gave up as designed. */
int pbf_selftest_bounded_wait(uint32_t spin_limit, void* d_scratch);

/* The same for the wait on a tile's shared-memory staging (TMA bulk copies
 * completing on an mbarrier): one block arms its barrier for bytes that no
 * copy delivers; after spin_limit polls it records the stage timeout and
 * returns.  d_scratch: caller-owned device memory of >= 4 bytes.  Returns
 * PBF_ERR_TIMEOUT when the wait gave up as designed. */
int pbf_selftest_stage_wait(uint32_t spin_limit, void* d_scratch);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* PBF_H */
