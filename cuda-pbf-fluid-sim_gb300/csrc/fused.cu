// fused.cu - the fused GB300 step.
//
// Phase order is the reference's (sim/phases.cpp:30-117,
// sim/post_ops.cpp:73-85, commit sim/simulator.cpp:144-159); kernels are
// fused where no global barrier separates them:
//   k_predict_keys   predict + boundary(e=0) + cell key          (ids)
//   radix sort       (key, id) -> (key_s, perm)
//   k_gather         re-predicts in cell order (bit-identical to the keyed
//                    prediction), stores step-start positions in cell order
//   cell tables      dense lower-bound table (+ compact table when hashed)
//   k_lambda         per iteration
//   k_delta          per iteration; the last one also applies the post-solve
//                    boundary (e=0) and computes v = (x - p)/dt
//   k_commit         XSPH (Jacobi) + boundary(e) + scatter back to ids
#include "fused.cuh"

#include "grid.cuh"
#include "pbf_common.cuh"
#include "sort.cuh"

namespace pbf {
namespace {

constexpr int kBS = 256;
// Neighbour kernels: 128 threads, a 32-entry neighbour queue per thread in
// shared memory (16 KB per block), column-major so a warp's queue writes hit
// 32 distinct banks.
constexpr int kNbrBS = 128;
constexpr int kQueue = 32;

__global__ void __launch_bounds__(kBS) k_predict_keys(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                      const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                      uint32_t* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const sim::GridBounds g = dpp->grid;
    const float4 x = predict_clamped(pos[i], vel[i], dpp->gravity, dpp->dt, g);
    keys[i] = cell_key(x, g);
}

__global__ void __launch_bounds__(kBS) k_gather(const uint32_t* __restrict__ perm, const float4* __restrict__ pos,
                                                const float4* __restrict__ vel,
                                                const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                float4* __restrict__ pred_s, float4* __restrict__ pos_s) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const uint32_t i = perm[s];
    const float4 p = pos[i];
    pred_s[s] = predict_clamped(p, vel[i], dpp->gravity, dpp->dt, dpp->grid);
    pos_s[s] = p;
}

__global__ void __launch_bounds__(kNbrBS) k_lambda(const float4* __restrict__ pred, const uint32_t* __restrict__ key_s,
                                                   const uint32_t* __restrict__ lb,
                                                   const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                   float* __restrict__ lam) {
    __shared__ uint32_t s_queue[kQueue * kNbrBS];
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = s < N;  // every lane takes part in the warp-wide rounds
    const uint32_t sc = active ? s : 0u;
    const sim::DeviceParams& dp = *dpp;
    int cx, cy, cz;
    decode_key(key_s[sc], dp.grid.dim, cx, cy, cz);
    const float l = lambda_queued<kQueue, kNbrBS>(active, sc, pred[sc], cx, cy, cz, dp, lb, pred, s_queue + threadIdx.x);
    if (active) lam[s] = l;
}

template <bool kLast>
__global__ void __launch_bounds__(kNbrBS) k_delta(const float4* __restrict__ pred, const float* __restrict__ lam,
                                                  const uint32_t* __restrict__ key_s, const uint32_t* __restrict__ lb,
                                                  const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                  float4* __restrict__ pred_out, const float4* __restrict__ pos_s,
                                                  float4* __restrict__ vel_s) {
    __shared__ uint32_t s_queue[kQueue * kNbrBS];
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = s < N;  // every lane takes part in the warp-wide rounds
    const uint32_t sc = active ? s : 0u;
    const sim::DeviceParams& dp = *dpp;
    int cx, cy, cz;
    decode_key(key_s[sc], dp.grid.dim, cx, cy, cz);
    const float4 pi = pred[sc];
    const float3 d = delta_queued<kQueue, kNbrBS>(active, sc, pi, lam[sc], cx, cy, cz, dp, scorr_wq(dp), lb, pred,
                                                   lam, s_queue + threadIdx.x);
    if (!active) return;
    float4 x = make_float4(add_(pi.x, d.x), add_(pi.y, d.y), add_(pi.z, d.z), pi.w);
    if (kLast) {
        // Boundary(e=0) after the solve loop (sim/phases.cpp:94); its velocity
        // half is overwritten by the velocity phase, so only x is clamped.
        float4 vdummy = make_float4(0.f, 0.f, 0.f, 0.f);
        boundary_apply(x, vdummy, dp.grid, 0.0f);
        // PhaseVelocity (sim/phases.cpp:102-105): v = (x - p) * (1/dt).
        const float inv_dt = div_(1.0f, dp.dt);
        const float4 p = pos_s[s];
        vel_s[s] = make_float4(mul_(sub_(x.x, p.x), inv_dt), mul_(sub_(x.y, p.y), inv_dt),
                               mul_(sub_(x.z, p.z), inv_dt), 0.0f);
    }
    pred_out[s] = x;
}

// solverIters == 0: the boundary and velocity phases on the prediction.
__global__ void __launch_bounds__(kBS) k_finalize_no_iters(float4* __restrict__ pred, const float4* __restrict__ pos_s,
                                                           const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                           float4* __restrict__ vel_s) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    float4 x = pred[s];
    float4 vdummy = make_float4(0.f, 0.f, 0.f, 0.f);
    boundary_apply(x, vdummy, dpp->grid, 0.0f);
    const float inv_dt = div_(1.0f, dpp->dt);
    const float4 p = pos_s[s];
    vel_s[s] = make_float4(mul_(sub_(x.x, p.x), inv_dt), mul_(sub_(x.y, p.y), inv_dt), mul_(sub_(x.z, p.z), inv_dt),
                           0.0f);
    pred[s] = x;
}

template <bool kXsph>
__global__ void __launch_bounds__(kNbrBS) k_commit(const float4* __restrict__ pred, const float4* __restrict__ vel_s,
                                                   const uint32_t* __restrict__ key_s, const uint32_t* __restrict__ lb,
                                                   const uint32_t* __restrict__ perm,
                                                   const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                   float4* __restrict__ pos, float4* __restrict__ vel) {
    __shared__ uint32_t s_queue[kXsph ? kQueue * kNbrBS : 1];
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = s < N;  // every lane takes part in the warp-wide rounds
    const uint32_t sc = active ? s : 0u;
    const sim::DeviceParams& dp = *dpp;
    float4 x = pred[sc];
    float4 v = vel_s[sc];
    if (kXsph && dp.xsph_c > 0.f) {
        int cx, cy, cz;
        decode_key(key_s[sc], dp.grid.dim, cx, cy, cz);
        v = xsph_queued<kQueue, kNbrBS>(active, sc, x, v, cx, cy, cz, dp, lb, pred, vel_s, s_queue + threadIdx.x);
    }
    if (!active) return;
    boundary_apply(x, v, dp.grid, dp.boundaryRestitution);
    const uint32_t i = perm[s];
    pos[i] = x;
    vel[i] = v;
}

__global__ void k_scatter_lambda(const float* __restrict__ lam_s, const uint32_t* __restrict__ perm, uint32_t N,
                                 float* __restrict__ out) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    out[perm[s]] = lam_s[s];
}

// ---------------------------------------------------------------- stats
__global__ void __launch_bounds__(kBS) k_position_keys(const float4* __restrict__ pos,
                                                       const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                       uint32_t* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    keys[i] = cell_key(pos[i], dpp->grid);
}

__global__ void __launch_bounds__(kBS) k_gather_positions(const uint32_t* __restrict__ perm,
                                                          const float4* __restrict__ pos, uint32_t N,
                                                          float4* __restrict__ out) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    out[s] = pos[perm[s]];
}

// Per-block partial sums of |C|, max|C|, max(C,0), neighbour count over a
// fixed slot range, reduced in a fixed tree order (deterministic).
__global__ void __launch_bounds__(kBS) k_density_partials(const float4* __restrict__ xs,
                                                          const uint32_t* __restrict__ key_s,
                                                          const uint32_t* __restrict__ lb,
                                                          const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                          uint32_t perBlock, double* __restrict__ partials) {
    const sim::DeviceParams& dp = *dpp;
    const sim::KernelCoeffs& kc = dp.kernel;
    double a = 0, m = 0, pc = 0, nb = 0;
    const uint32_t beg = blockIdx.x * perBlock;
    const uint32_t end = min(N, beg + perBlock);
    for (uint32_t s = beg + threadIdx.x; s < end; s += blockDim.x) {
        int cx, cy, cz;
        decode_key(key_s[s], dp.grid.dim, cx, cy, cz);
        const float4 pi = xs[s];
        float rho = 0.f;
        int cnt = 0;
        walk_neighbours(cx, cy, cz, neighbour_reach(dp), dp.grid.dim, LbRows{lb}, [&](uint32_t k) -> bool {
            if (k == s) return true;
            const float4 pj = __ldg(xs + k);
            const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            const float r2 = rx * rx + ry * ry + rz * rz;
            if (r2 > kc.h2) return true;
            const float hr2 = kc.h2 - r2;
            rho += dp.particleMass * kc.poly6 * hr2 * hr2 * hr2;
            ++cnt;
            return true;
        });
        const double C = (dp.restDensity > 0.f) ? double(rho) / double(dp.restDensity) - 1.0 : 0.0;
        a += fabs(C);
        m = fmax(m, fabs(C));
        pc += C > 0 ? C : 0.0;
        nb += cnt;
    }
    __shared__ double sh[4][kBS];
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = m;
    sh[2][threadIdx.x] = pc;
    sh[3][threadIdx.x] = nb;
    __syncthreads();
    for (int w = kBS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
            sh[1][threadIdx.x] = fmax(sh[1][threadIdx.x], sh[1][threadIdx.x + w]);
            sh[2][threadIdx.x] += sh[2][threadIdx.x + w];
            sh[3][threadIdx.x] += sh[3][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[4 * blockIdx.x + 0] = sh[0][0];
        partials[4 * blockIdx.x + 1] = sh[1][0];
        partials[4 * blockIdx.x + 2] = sh[2][0];
        partials[4 * blockIdx.x + 3] = sh[3][0];
    }
}

__global__ void k_density_final(const double* __restrict__ partials, unsigned nblocks, uint32_t N,
                                 double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0, m = 0, pc = 0, nb = 0;
    for (unsigned b = 0; b < nblocks; ++b) {
        a += partials[4 * b + 0];
        m = fmax(m, partials[4 * b + 1]);
        pc += partials[4 * b + 2];
        nb += partials[4 * b + 3];
    }
    const double n = N ? double(N) : 1.0;
    out[0] = a / n;
    out[1] = m;
    out[2] = pc / n;
    out[3] = nb / n;
}

}  // namespace

cudaError_t fused_predict_keys(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    if (sh.N == 0) return cudaSuccess;
    k_predict_keys<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.pos, b.vel, b.dp, sh.N, b.keys);
    return cudaGetLastError();
}

cudaError_t fused_sort(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    return sort_pairs(b.sort_temp, b.sort_bytes, b.keys, b.key_s, nullptr, b.perm, sh.N, sh.key_bits, s, b.err);
}

cudaError_t fused_gather_and_tables(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    if (sh.N > 0) k_gather<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.perm, b.pos, b.vel, b.dp, sh.N, b.pred_a, b.pos_s);
    cudaError_t e = launch_cell_lb(b.lb, b.key_s, sh.N, sh.numCells, s);
    if (e != cudaSuccess) return e;
    if (sh.hashed) {
        e = launch_compact(b.compact_temp, b.compact_bytes, b.uk, b.off, b.count, nullptr, b.key_s, sh.N, s, b.err);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

cudaError_t fused_solve_phase(const FusedBufs& b, const FusedShape& sh, int it, int which, cudaStream_t s) {
    if (sh.N == 0 || it < 0 || it >= sh.iters) return cudaSuccess;
    const unsigned g = blocks_for(sh.N, kNbrBS);
    // iteration it reads buffer (it even ? a : b) and writes the other one
    float4* cur = (it % 2 == 0) ? b.pred_a : b.pred_b;
    float4* nxt = (it % 2 == 0) ? b.pred_b : b.pred_a;
    if (which == 0) {
        k_lambda<<<g, kNbrBS, 0, s>>>(cur, b.key_s, b.lb, b.dp, sh.N, b.lam_s);
    } else if (it == sh.iters - 1) {
        k_delta<true><<<g, kNbrBS, 0, s>>>(cur, b.lam_s, b.key_s, b.lb, b.dp, sh.N, nxt, b.pos_s, b.vel_s);
    } else {
        k_delta<false><<<g, kNbrBS, 0, s>>>(cur, b.lam_s, b.key_s, b.lb, b.dp, sh.N, nxt, b.pos_s, b.vel_s);
    }
    return cudaGetLastError();
}

cudaError_t fused_solve(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    if (sh.N == 0) return cudaSuccess;
    for (int it = 0; it < sh.iters; ++it) {
        fused_solve_phase(b, sh, it, 0, s);
        fused_solve_phase(b, sh, it, 1, s);
    }
    if (sh.iters <= 0)
        k_finalize_no_iters<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.pred_a, b.pos_s, b.dp, sh.N, b.vel_s);
    return cudaGetLastError();
}

cudaError_t fused_commit(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    if (sh.N == 0) return cudaSuccess;
    const float4* x = fused_final_pred(b, sh);
    const unsigned g = blocks_for(sh.N, kNbrBS);
    if (sh.xsph)
        k_commit<true><<<g, kNbrBS, 0, s>>>(x, b.vel_s, b.key_s, b.lb, b.perm, b.dp, sh.N, b.pos, b.vel);
    else
        k_commit<false><<<g, kNbrBS, 0, s>>>(x, b.vel_s, b.key_s, b.lb, b.perm, b.dp, sh.N, b.pos, b.vel);
    return cudaGetLastError();
}

cudaError_t fused_scatter_lambda(const FusedBufs& b, const FusedShape& sh, float* lambda_by_id, cudaStream_t s) {
    if (sh.N == 0) return cudaSuccess;
    k_scatter_lambda<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.lam_s, b.perm, sh.N, lambda_by_id);
    return cudaGetLastError();
}

cudaError_t fused_density_stats(const FusedBufs& b, const FusedShape& sh, cudaStream_t s) {
    if (sh.N == 0) return cudaMemsetAsync(b.stats_out, 0, 4 * sizeof(double), s);
    // Fresh grid over the committed positions (keys -> sort -> lb), using the
    // step's sorted buffers as scratch.
    k_position_keys<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.pos, b.dp, sh.N, b.keys);
    cudaError_t e = sort_pairs(b.sort_temp, b.sort_bytes, b.keys, b.key_s, nullptr, b.perm, sh.N, sh.key_bits, s, b.err);
    if (e != cudaSuccess) return e;
    k_gather_positions<<<blocks_for(sh.N, kBS), kBS, 0, s>>>(b.perm, b.pos, sh.N, b.pred_b);
    e = launch_cell_lb(b.lb, b.key_s, sh.N, sh.numCells, s);
    if (e != cudaSuccess) return e;
    unsigned nb = blocks_for(sh.N, 1024u);
    if (nb > kStatsMaxBlocks) nb = kStatsMaxBlocks;
    const uint32_t perBlock = (sh.N + nb - 1) / nb;
    k_density_partials<<<nb, kBS, 0, s>>>(b.pred_b, b.key_s, b.lb, b.dp, sh.N, perBlock, b.stats_partials);
    k_density_final<<<1, 32, 0, s>>>(b.stats_partials, nb, sh.N, b.stats_out);
    return cudaGetLastError();
}

}  // namespace pbf
