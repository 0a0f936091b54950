// phases.cu - reference-layout phase kernels.
//
// One thread per sorted slot, like the reference; the neighbour math is the
// shared restatement in pbf_common.cuh and each (dz,dy) row of the stencil is
// walked as one contiguous slot range.
#include "phases.cuh"

#include "pbf_common.cuh"

namespace pbf {
namespace {

constexpr int kBS = 256;

// sim/integrate.cu:29-52 (position predict only; w kept).
__global__ void k_integrate_ref(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                float4* __restrict__ pred, float3 g, float dt, uint32_t N) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float4 p = pos[i], v = vel[i];
    const float vx = __fmaf_rn(g.x, dt, v.x);
    const float vy = __fmaf_rn(g.y, dt, v.y);
    const float vz = __fmaf_rn(g.z, dt, v.z);
    pred[i] = make_float4(__fmaf_rn(vx, dt, p.x), __fmaf_rn(vy, dt, p.y), __fmaf_rn(vz, dt, p.z), p.w);
}

__global__ void k_boundary_ref(float4* __restrict__ pred, float4* __restrict__ vel, sim::GridBounds g, float e,
                               uint32_t N) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    float4 p = pred[i], v = vel[i];
    boundary_apply(p, v, g, e);
    pred[i] = p;
    vel[i] = v;
}

__global__ void k_velocity_ref(float4* __restrict__ vel, const float4* __restrict__ pos,
                               const float4* __restrict__ pred, float inv_dt, uint32_t N) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float4 p = pos[i], q = pred[i];
    vel[i] = make_float4((q.x - p.x) * inv_dt, (q.y - p.y) * inv_dt, (q.z - p.z) * inv_dt, 0.0f);
}

template <class Rows>
__device__ __forceinline__ void lambda_ref_body(float* lambda, const float4* __restrict__ pred,
                                                const uint32_t* __restrict__ idx, const uint32_t* __restrict__ keys,
                                                const sim::DeviceParams& dp, uint32_t N, Rows rows) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const uint32_t i = idx[s];
    int cx, cy, cz;
    decode_key(keys[s], dp.grid.dim, cx, cy, cz);
    lambda[i] = lambda_of(i, pred[i], cx, cy, cz, dp, rows, [&](uint32_t k, uint32_t& j) {
        j = __ldg(idx + k);
        return __ldg(pred + j);
    });
}

__global__ void k_lambda_dense(float* lambda, const float4* __restrict__ pred, const uint32_t* __restrict__ idx,
                               const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                               const uint32_t* __restrict__ end, sim::DeviceParams dp, uint32_t N) {
    lambda_ref_body(lambda, pred, idx, keys, dp, N, DenseRows{start, end});
}

__global__ void k_lambda_compact(float* lambda, const float4* __restrict__ pred, const uint32_t* __restrict__ idx,
                                 const uint32_t* __restrict__ keys, const uint32_t* __restrict__ uk,
                                 const uint32_t* __restrict__ off, const uint32_t* __restrict__ count,
                                 sim::DeviceParams dp, uint32_t N) {
    lambda_ref_body(lambda, pred, idx, keys, dp, N, CompactRows{uk, off, min(*count, N)});
}

template <class Rows>
__device__ __forceinline__ void delta_ref_body(float4* delta, const float4* __restrict__ pred,
                                               const float* __restrict__ lambda, const uint32_t* __restrict__ idx,
                                               const uint32_t* __restrict__ keys, const sim::DeviceParams& dp,
                                               uint32_t N, Rows rows) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const uint32_t i = idx[s];
    int cx, cy, cz;
    decode_key(keys[s], dp.grid.dim, cx, cy, cz);
    const float3 d = delta_of(i, pred[i], lambda[i], cx, cy, cz, dp, scorr_wq(dp), rows,
                              [&](uint32_t k, uint32_t& j, float& lj) {
                                  j = __ldg(idx + k);
                                  lj = __ldg(lambda + j);
                                  return __ldg(pred + j);
                              });
    delta[i] = make_float4(d.x, d.y, d.z, 0.0f);
}

__global__ void k_delta_dense(float4* delta, const float4* __restrict__ pred, const float* __restrict__ lambda,
                              const uint32_t* __restrict__ idx, const uint32_t* __restrict__ keys,
                              const uint32_t* __restrict__ start, const uint32_t* __restrict__ end,
                              sim::DeviceParams dp, uint32_t N) {
    delta_ref_body(delta, pred, lambda, idx, keys, dp, N, DenseRows{start, end});
}

__global__ void k_delta_compact(float4* delta, const float4* __restrict__ pred, const float* __restrict__ lambda,
                                const uint32_t* __restrict__ idx, const uint32_t* __restrict__ keys,
                                const uint32_t* __restrict__ uk, const uint32_t* __restrict__ off,
                                const uint32_t* __restrict__ count, sim::DeviceParams dp, uint32_t N) {
    delta_ref_body(delta, pred, lambda, idx, keys, dp, N, CompactRows{uk, off, min(*count, N)});
}

// sim/pbf_delta_apply.cu:223-235 (KApplyDelta).
__global__ void k_apply_delta(float4* __restrict__ pred, const float4* __restrict__ delta,
                              const uint32_t* __restrict__ idx, uint32_t N) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const uint32_t i = idx[s];
    const float4 d = delta[i], b = pred[i];
    pred[i] = make_float4(b.x + d.x, b.y + d.y, b.z + d.z, b.w);
}

template <class Rows>
__device__ __forceinline__ void xsph_ref_body(float4* vel_out, const float4* __restrict__ vel_in,
                                              const float4* __restrict__ pred, const uint32_t* __restrict__ idx,
                                              const uint32_t* __restrict__ keys, const sim::DeviceParams& dp,
                                              uint32_t N, Rows rows) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const uint32_t i = idx[s];
    int cx, cy, cz;
    decode_key(keys[s], dp.grid.dim, cx, cy, cz);
    vel_out[i] = xsph_of(i, pred[i], vel_in[i], cx, cy, cz, dp, rows, [&](uint32_t k, uint32_t& j, float4& vj) {
        j = __ldg(idx + k);
        vj = __ldg(vel_in + j);
        return __ldg(pred + j);
    });
}

__global__ void k_xsph_dense(float4* vel_out, const float4* __restrict__ vel_in, const float4* __restrict__ pred,
                             const uint32_t* __restrict__ idx, const uint32_t* __restrict__ keys,
                             const uint32_t* __restrict__ start, const uint32_t* __restrict__ end,
                             sim::DeviceParams dp, uint32_t N) {
    xsph_ref_body(vel_out, vel_in, pred, idx, keys, dp, N, DenseRows{start, end});
}

__global__ void k_xsph_compact(float4* vel_out, const float4* __restrict__ vel_in, const float4* __restrict__ pred,
                               const uint32_t* __restrict__ idx, const uint32_t* __restrict__ keys,
                               const uint32_t* __restrict__ uk, const uint32_t* __restrict__ off,
                               const uint32_t* __restrict__ count, sim::DeviceParams dp, uint32_t N) {
    xsph_ref_body(vel_out, vel_in, pred, idx, keys, dp, N, CompactRows{uk, off, min(*count, N)});
}

}  // namespace

cudaError_t launch_integrate_pred_ref(const float4* pos, const float4* vel, float4* pred, float3 g, float dt,
                                      uint32_t N, cudaStream_t s) {
    if (N == 0) return cudaSuccess;
    k_integrate_ref<<<blocks_for(N, kBS), kBS, 0, s>>>(pos, vel, pred, g, dt, N);
    return cudaGetLastError();
}

cudaError_t launch_boundary_ref(float4* pred, float4* vel, const sim::GridBounds& g, float restitution, uint32_t N,
                                cudaStream_t s) {
    if (N == 0) return cudaSuccess;
    k_boundary_ref<<<blocks_for(N, kBS), kBS, 0, s>>>(pred, vel, g, restitution, N);
    return cudaGetLastError();
}

cudaError_t launch_velocity_ref(float4* vel, const float4* pos, const float4* pred, float inv_dt, uint32_t N,
                                cudaStream_t s) {
    if (N == 0) return cudaSuccess;
    k_velocity_ref<<<blocks_for(N, kBS), kBS, 0, s>>>(vel, pos, pred, inv_dt, N);
    return cudaGetLastError();
}

cudaError_t launch_lambda_ref(float* lambda, const float4* pred, const uint32_t* idx, const uint32_t* keys,
                              const RefTable& t, const sim::DeviceParams& dp, uint32_t N, cudaStream_t s) {
    if (N == 0) return cudaSuccess;
    if (t.unique_keys)
        k_lambda_compact<<<blocks_for(N, kBS), kBS, 0, s>>>(lambda, pred, idx, keys, t.unique_keys, t.offsets,
                                                            t.count, dp, N);
    else
        k_lambda_dense<<<blocks_for(N, kBS), kBS, 0, s>>>(lambda, pred, idx, keys, t.start, t.end, dp, N);
    return cudaGetLastError();
}

cudaError_t launch_delta_apply_ref(float4* pred, float4* delta, const float* lambda, const uint32_t* idx,
                                   const uint32_t* keys, const RefTable& t, const sim::DeviceParams& dp, uint32_t N,
                                   cudaStream_t s) {
    if (N == 0) return cudaSuccess;
    if (t.unique_keys)
        k_delta_compact<<<blocks_for(N, kBS), kBS, 0, s>>>(delta, pred, lambda, idx, keys, t.unique_keys, t.offsets,
                                                           t.count, dp, N);
    else
        k_delta_dense<<<blocks_for(N, kBS), kBS, 0, s>>>(delta, pred, lambda, idx, keys, t.start, t.end, dp, N);
    k_apply_delta<<<blocks_for(N, kBS), kBS, 0, s>>>(pred, delta, idx, N);
    return cudaGetLastError();
}

cudaError_t launch_xsph_ref(float4* vel_out, const float4* vel_in, const float4* pred, const uint32_t* idx,
                            const uint32_t* keys, const RefTable& t, const sim::DeviceParams& dp, uint32_t N,
                            cudaStream_t s) {
    if (N == 0 || !(dp.xsph_c > 0.f)) return cudaSuccess;
    if (t.unique_keys)
        k_xsph_compact<<<blocks_for(N, kBS), kBS, 0, s>>>(vel_out, vel_in, pred, idx, keys, t.unique_keys, t.offsets,
                                                          t.count, dp, N);
    else
        k_xsph_dense<<<blocks_for(N, kBS), kBS, 0, s>>>(vel_out, vel_in, pred, idx, keys, t.start, t.end, dp, N);
    return cudaGetLastError();
}

}  // namespace pbf
