// launch_abi.h - the reference's own extern "C" launcher symbols.
//
// libpbf_gb300 exports these exact names and signatures, so a build of the
// reference can link the library in place of compiling sim/*.cu: the
// prototypes below are the ones the reference declares at sim/phases.cpp:8-25,
// sim/simulator.cpp:38-65 and sim/post_ops.cpp:8-10.  Differences in
// behaviour, all deliberate:
//   * LaunchLambda/LaunchLambdaCompact write `lambda` and read `pos_pred`
//     from their arguments; the reference ignores both and goes through the
//     device globals g_lambda / g_pos_pred (sim/pbf_lambda.cu:256,272), which
//     it binds to the same two buffers.
//   * LaunchXSPH/LaunchXSPHCompact with vel_out == vel_in (how the reference
//     calls them, sim/post_ops.cpp:59,65) read a stream-ordered snapshot of
//     the old velocities (cudaMallocAsync/cudaFreeAsync), i.e. the Jacobi
//     update, instead of racing on the array being written.
//   * LaunchSortPairs sorts with this library's onesweep radix sort; temp
//     sizes come from LaunchSortPairsQuery as before.
//   * LaunchCellRangesCompact keeps process-global scratch like the reference
//     (sim/cell_compact.cu:50-93); EnsureCellCompactScratch sizes it.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "parameters.h"

extern "C" {
// sim/integrate.cu:76-89
void LaunchIntegratePred(float4* posCurr, const float4* velSrc, float4* posPred, float3 gravity, float dt, uint32_t N,
                         cudaStream_t s);
// sim/boundary.cu:37-40
void LaunchBoundary(float4* pos_pred, float4* vel, sim::GridBounds grid, float restitution, uint32_t N,
                    cudaStream_t s);
// sim/boundary.cu:41-44
void LaunchVelocity(float4* vel, const float4* pos, const float4* pos_pred, float inv_dt, uint32_t N,
                    cudaStream_t s);
// sim/hash_keys.cu:30-34
void LaunchHashKeys(uint32_t* keys, uint32_t* indices, const float4* pos, sim::GridBounds grid, uint32_t N,
                    cudaStream_t s);
// sim/sort_pairs.cu:5-16
void LaunchSortPairsQuery(size_t* tempBytes, const uint32_t* d_keys_in, uint32_t* d_keys_out,
                          const uint32_t* d_vals_in, uint32_t* d_vals_out, uint32_t N, cudaStream_t s);
// sim/sort_pairs.cu:18-27
void LaunchSortPairs(void* d_temp_storage, size_t tempBytes, uint32_t* d_keys_in, uint32_t* d_keys_out,
                     uint32_t* d_vals_in, uint32_t* d_vals_out, uint32_t N, cudaStream_t s);
// sim/cell_ranges.cu:55-80
void LaunchCellRanges(uint32_t* cellStart, uint32_t* cellEnd, const uint32_t* keysSorted, uint32_t N,
                      uint32_t numCells, cudaStream_t s);
// sim/cell_compact.cu:58-93
bool EnsureCellCompactScratch(uint32_t N, uint32_t threadsPerBlock);
// sim/cell_compact.cu:187-231
void LaunchCellRangesCompact(uint32_t* d_uniqueKeys, uint32_t* d_offsets, uint32_t* d_compactCount,
                             const uint32_t* d_keysSorted, uint32_t N, cudaStream_t s);
// sim/pbf_lambda.cu:246-258
void LaunchLambda(float* lambda, const float4* pos_pred, const uint32_t* indicesSorted, const uint32_t* keysSorted,
                  const uint32_t* cellStart, const uint32_t* cellEnd, sim::DeviceParams dp, uint32_t N,
                  cudaStream_t s);
// sim/pbf_lambda.cu:260-274
void LaunchLambdaCompact(float* lambda, const float4* pos_pred, const uint32_t* indicesSorted,
                         const uint32_t* keysSorted, const uint32_t* uniqueKeys, const uint32_t* offsets,
                         const uint32_t* compactCount, sim::DeviceParams dp, uint32_t N, cudaStream_t s);
// sim/pbf_delta_apply.cu:239-258
void LaunchDeltaApply(float4* pos_pred, float4* delta, const float* lambda, const uint32_t* indicesSorted,
                      const uint32_t* keysSorted, const uint32_t* cellStart, const uint32_t* cellEnd,
                      sim::DeviceParams dp, uint32_t N, cudaStream_t s);
// sim/pbf_delta_apply.cu:260-280
void LaunchDeltaApplyCompact(float4* pos_pred, float4* delta, const float* lambda, const uint32_t* indicesSorted,
                             const uint32_t* keysSorted, const uint32_t* uniqueKeys, const uint32_t* offsets,
                             const uint32_t* compactCount, sim::DeviceParams dp, uint32_t N, cudaStream_t s);
// sim/xsph.cu:189-205
void LaunchXSPH(float4* vel_out, const float4* vel_in, const float4* pos_pred, const uint32_t* indicesSorted,
                const uint32_t* keysSorted, const uint32_t* cellStart, const uint32_t* cellEnd, sim::DeviceParams dp,
                uint32_t N, cudaStream_t s);
// sim/xsph.cu:207-228
void LaunchXSPHCompact(float4* vel_out, const float4* vel_in, const float4* pos_pred, const uint32_t* indicesSorted,
                       const uint32_t* keysSorted, const uint32_t* uniqueKeys, const uint32_t* offsets,
                       const uint32_t* compactCount, sim::DeviceParams dp, uint32_t N, cudaStream_t s);
}
