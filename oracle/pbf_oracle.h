/*
 * pbf_oracle.h - CPU restatement of PBF-X's per-step simulation math.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU kernels
 * of libpbf_gb300: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline may load it.  Nothing in the product links or calls it.
 *
 * Each function restates one reference CUDA kernel (file:line cited at the
 * definition) as a sequential/OpenMP CPU loop over the same indices, in the
 * same neighbour order (dz, dy, dx outer; sorted order inner), so FP32
 * results agree with the GPU to rounding (nvcc contracts a*b+c into FMA; the
 * oracle does not, except in the predict step where the GPU uses an explicit
 * FMA, mirrored here with fmaf so that cell keys are bit-exact).
 *
 * Pinning: the reference ships no tests, fixtures or CPU PBF code
 * (README.md:85, sim/kernel_fallback.cpp is a vector add).  The oracle is
 * pinned by (a) hand-derived known-answer cases in tests/golden/ and (b) the
 * reference's own CUDA kernels, compiled from source for sm_103a and run on
 * the GPU, whose outputs are committed as fixtures by
 * oracle/ref/make_ref_fixtures.py.
 *
 * XSPH is the Jacobi form (old velocities in, new out); the reference runs it
 * in place (sim/post_ops.cpp:59,65), which is a data race.
 */
#ifndef PBF_ORACLE_H
#define PBF_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/pbf/pbf_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Optional per-step intermediates (each pointer may be NULL). */
typedef struct oracle_trace {
    uint32_t* keys;         /* [N] cell key of each particle (id order) */
    uint32_t* keys_sorted;  /* [N] */
    uint32_t* perm;         /* [N] indices_sorted */
    uint32_t* cell_start;   /* [numCells] dense format (dense mode) */
    uint32_t* cell_end;     /* [numCells] */
    uint32_t* unique_keys;  /* [N] compact format (hashed mode) */
    uint32_t* offsets;      /* [N+1] */
    uint32_t* compact_count;/* [1] */
    float*    lambda;       /* [N] last iteration's lambda (id order) */
    float4*   pred_solved;  /* [N] pred after the last delta-apply, before the boundary */
    float4*   vel_pre_xsph; /* [N] velocity after the velocity phase */
} oracle_trace;

int  oracle_num_threads(void);
void oracle_set_num_threads(int n);

void oracle_integrate_pred(const float4* pos, const float4* vel, float4* pred,
                           float3 gravity, float dt, uint32_t N);
void oracle_boundary(float4* pred, float4* vel, const pbf_grid_bounds* g,
                     float restitution, uint32_t N);
void oracle_velocity(float4* vel, const float4* pos, const float4* pred,
                     float inv_dt, uint32_t N);
void oracle_hash_keys(uint32_t* keys, uint32_t* indices, const float4* pred,
                      const pbf_grid_bounds* g, uint32_t N);
void oracle_sort_pairs(const uint32_t* keys_in, uint32_t* keys_out,
                       const uint32_t* vals_in, uint32_t* vals_out, uint32_t N);
void oracle_cell_ranges(uint32_t* start, uint32_t* end, const uint32_t* keys_sorted,
                        uint32_t N, uint32_t numCells);
void oracle_cell_ranges_compact(uint32_t* unique_keys, uint32_t* offsets,
                                uint32_t* count, const uint32_t* keys_sorted, uint32_t N);

/* Neighbour phases; table = dense (start/end) when unique_keys == NULL,
 * compact (unique_keys/offsets/count) otherwise. */
typedef struct oracle_table {
    const uint32_t* start;
    const uint32_t* end;
    const uint32_t* unique_keys;
    const uint32_t* offsets;
    uint32_t count;
} oracle_table;

void oracle_lambda(float* lambda, const float4* pred, const uint32_t* idx_sorted,
                   const uint32_t* keys_sorted, const oracle_table* t,
                   const pbf_device_params* dp, uint32_t N);
void oracle_delta_apply(float4* pred, float4* delta, const float* lambda,
                        const uint32_t* idx_sorted, const uint32_t* keys_sorted,
                        const oracle_table* t, const pbf_device_params* dp, uint32_t N);
void oracle_xsph(float4* vel_out, const float4* vel_in, const float4* pred,
                 const uint32_t* idx_sorted, const uint32_t* keys_sorted,
                 const oracle_table* t, const pbf_device_params* dp, uint32_t N);

/* One full step in FP32, reference phase order (sim/phases.cpp:30-117,
 * sim/post_ops.cpp:73-85) plus the commit pos <- pred
 * (sim/simulator.cpp:144-159).  pos/vel are updated in place. */
int oracle_step_f32(const pbf_sim_params* p, int hashed, float4* pos, float4* vel,
                    uint32_t N, oracle_trace* trace);
/* Same step in FP64 (state as double[4*N], xyzw). */
int oracle_step_f64(const pbf_sim_params* p, int hashed, double* pos4, double* vel4,
                    uint32_t N);

/* Density-constraint statistics evaluated in FP64 on the given positions
 * (float4 or double4): out[0] mean |C|, out[1] max |C|, out[2] mean max(C,0),
 * out[3] mean neighbour count; C_i = rho_i/rho0 - 1 with
 * rho_i = sum_{j != i, r^2 <= h^2} m W_poly6, uncapped. */
void oracle_density_stats_f32pos(const pbf_sim_params* p, const float4* pos,
                                 uint32_t N, double out[4]);
void oracle_density_stats_f64pos(const pbf_sim_params* p, const double* pos4,
                                 uint32_t N, double out[4]);

/* Steps differentiated in forward mode (dual numbers, derivative part in
 * FP64): pos4/vel4 (double[4N], xyzw) are advanced `steps` steps in place, and
 * the direction (dpos4, dvel4, dxsph_c) of the initial state is carried
 * along, so that on return dpos4/dvel4 hold the directional derivative of the
 * final state.  Branches (neighbour sets, caps, clamps, boundary) follow the
 * values.  fp32_values = 0: the values are the FP64 step's; 1: the values are
 * the FP32 oracle step's (pos4/vel4 then hold floats), so the derivative is
 * taken along the FP32 trajectory the GPU computes - the reference tape of
 * the adjoint's vector-Jacobian products. */
int oracle_step_jvp(const pbf_sim_params* p, int hashed, int fp32_values, double* pos4,
                    double* vel4, double* dpos4, double* dvel4, double dxsph_c, uint32_t N,
                    int steps);

/* Scene generation for the CPU arm, so that it needs no product library.
 * The dam-break parameters: particle radius 0.005 m, spacing 2r, h = 2.5 r
 * (engine/core/console.cpp:198-267), mass 1000 spacing^3, dt 1/120,
 * gravity -9.8 y, maxNeighbors 64, restitution 0, s_corr k 0.1 n 4
 * dq 0.2 h, lambda eps 100, XSPH 0.01, the other tuning fields at their
 * sim/parameters.h defaults, rho0 = the lambda-kernel density of an interior
 * particle of the unjittered lattice (its 6 face neighbours), grid [0,b] with
 * cell size h.  Returns 0, or 1 for an invalid box / iteration count. */
int oracle_dam_break_params(float bx, float by, float bz, int solver_iters,
                            uint32_t num_particles, pbf_sim_params* out);
/* nx*ny*nz particles at origin + index*spacing (x fastest), each axis
 * jittered by (2u - 1)*jitter with u = (mt19937_64 output >> 11) / 2^53,
 * three draws per particle in x, y, z order, clamped to the box, w = 1. */
void oracle_seed_lattice(float4* out, uint32_t nx, uint32_t ny, uint32_t nz, float ox,
                         float oy, float oz, float spacing, float jitter, uint64_t seed,
                         const pbf_grid_bounds* box);

#ifdef __cplusplus
}
#endif
#endif
