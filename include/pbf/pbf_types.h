/*
 * pbf_types.h - plain-C mirror of the PBF-X parameter structs.
 *
 * These structs have the same field order, types and sizes as the reference's
 * C++ structs in sim/parameters.h (KernelCoeffs 9-16, GridBounds 19-24,
 * PbfTuning 27-57, SimParams 60-77, DeviceParams 80-92).  The reference passes
 * sim::GridBounds and sim::DeviceParams *by value* across its extern "C"
 * launchers (e.g. sim/hash_keys.cu:30, sim/pbf_lambda.cu:246), so the C ABI of
 * a drop-in replacement is fixed by this layout.  include/pbf/parameters.h
 * static_asserts that the C++ sim:: structs and these C structs agree.
 *
 * Vector members use CUDA's C vector types (float3 / int3 / float4), which are
 * plain C structs of 4-byte members.
 */
#ifndef PBF_TYPES_H
#define PBF_TYPES_H

#include <stdint.h>
#include <vector_types.h> /* float3, float4, int3 (C-compatible) */

#ifdef __cplusplus
extern "C" {
#endif

/* Smoothing-kernel constants (reference sim/parameters.h:9-16). */
typedef struct pbf_kernel_coeffs {
    float h;
    float inv_h;
    float h2;
    float poly6; /* 315 / (64 pi h^9) */
    float spiky; /* 15 / (pi h^6) */
    float visc;  /* 15 / (2 pi h^3) */
} pbf_kernel_coeffs;

/* Axis-aligned container and its uniform grid (sim/parameters.h:19-24). */
typedef struct pbf_grid_bounds {
    float3 mins;
    float3 maxs;
    float  cellSize;
    int3   dim;
} pbf_grid_bounds;

/* PBF tuning block (sim/parameters.h:27-57); defaults in pbf_default_tuning(). */
typedef struct pbf_tuning {
    int   scorr_enable;
    float scorr_k;
    float scorr_n;
    float scorr_dq_h;
    float wq_min;
    float scorr_min;
    float grad_r_eps;
    float lambda_denom_eps;
    float compliance;
    int   xpbd_enable;
    int   enable_lambda_clamp;
    float lambda_max_abs;
    int   enable_disp_clamp;
    float disp_clamp_max_h;
    int   enable_relax;
    float relax_omega;
    int   xsph_gate_enable;
    int   xsph_n_min;
    int   xsph_n_max;
    int   lambda_warm_start_enable;
    float lambda_warm_start_decay;
    int   semi_implicit_integration_enable;
} pbf_tuning;

/* Host-side parameter aggregate (sim/parameters.h:60-77). */
typedef struct pbf_sim_params {
    uint32_t numParticles;
    uint32_t maxParticles;
    float3   gravity;
    float    dt;
    float    cfl;
    float    restDensity;
    int      solverIters;
    int      maxNeighbors;
    int      sortEveryN;
    float    boundaryRestitution;
    float    particleMass;
    pbf_tuning pbf;
    float    xsph_c;
    pbf_kernel_coeffs kernel;
    pbf_grid_bounds   grid;
    uint32_t ghostParticleCount;
} pbf_sim_params;

/* Device-side parameter snapshot (sim/parameters.h:80-92). */
typedef struct pbf_device_params {
    pbf_kernel_coeffs kernel;
    pbf_grid_bounds   grid;
    float3 gravity;
    float  restDensity;
    float  dt;
    float  inv_dt;
    float  boundaryRestitution;
    int    maxNeighbors;
    float  particleMass;
    pbf_tuning pbf;
    float  xsph_c;
} pbf_device_params;

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* PBF_TYPES_H */
