// ref_globals_shim.cuh - definitions of the reference's device-global
// pointer symbols (declared in the reference's sim/device_globals.cuh:8-15).
//
// TEST INFRASTRUCTURE ONLY.  The reference defines them in
// sim/device_globals.cu, whose include chain reaches <windows.h>; this shim is
// force-included when building the reference's pbf_lambda.cu into a
// stand-alone device image, so that KLambdaGlobals* (which read g_pos_pred and
// write g_lambda) can be driven from the harness.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sim {
struct Half4 {
    unsigned short x, y, z, w;
};
__device__ float4* g_pos = nullptr;
__device__ float4* g_vel = nullptr;
__device__ float4* g_pos_pred = nullptr;
__device__ float4* g_delta = nullptr;
__device__ float* g_lambda = nullptr;
__device__ uint32_t g_ghostCount = 0;
__device__ Half4* g_pos_h4 = nullptr;
__device__ Half4* g_vel_h4 = nullptr;
__device__ Half4* g_pos_pred_h4 = nullptr;
}  // namespace sim
