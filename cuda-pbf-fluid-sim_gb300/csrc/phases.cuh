// phases.cuh - reference-layout phase kernels (host launch helpers).
//
// Buffers follow the reference's DeviceBuffers / GridBuffers layout: particle
// arrays indexed by the original particle id, neighbour walks through
// indicesSorted.  Each helper mirrors one reference launcher.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pbf/parameters.h"

namespace pbf {

struct RefTable {
    // dense: start/end non-null; compact: unique_keys/offsets/count non-null
    const uint32_t* start;
    const uint32_t* end;
    const uint32_t* unique_keys;
    const uint32_t* offsets;
    const uint32_t* count;  // device pointer to M
};

cudaError_t launch_integrate_pred_ref(const float4* pos, const float4* vel, float4* pred, float3 g, float dt,
                                      uint32_t N, cudaStream_t s);
cudaError_t launch_boundary_ref(float4* pred, float4* vel, const sim::GridBounds& g, float restitution, uint32_t N,
                                cudaStream_t s);
cudaError_t launch_velocity_ref(float4* vel, const float4* pos, const float4* pred, float inv_dt, uint32_t N,
                                cudaStream_t s);
cudaError_t launch_lambda_ref(float* lambda, const float4* pred, const uint32_t* idx_sorted,
                              const uint32_t* keys_sorted, const RefTable& t, const sim::DeviceParams& dp,
                              uint32_t N, cudaStream_t s);
cudaError_t launch_delta_apply_ref(float4* pred, float4* delta, const float* lambda, const uint32_t* idx_sorted,
                                   const uint32_t* keys_sorted, const RefTable& t, const sim::DeviceParams& dp,
                                   uint32_t N, cudaStream_t s);
cudaError_t launch_xsph_ref(float4* vel_out, const float4* vel_in, const float4* pred, const uint32_t* idx_sorted,
                            const uint32_t* keys_sorted, const RefTable& t, const sim::DeviceParams& dp, uint32_t N,
                            cudaStream_t s);

}  // namespace pbf
