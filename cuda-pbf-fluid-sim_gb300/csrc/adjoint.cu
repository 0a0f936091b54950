// adjoint.cu - reverse-mode gradients of the PBF step.
//
// No counterpart in the reference.  pbf_forward runs a handle's scene for n
// steps and keeps (pos, vel) checkpoints every k steps; pbf_backward takes
// dL/d(final pos, final vel) and returns dL/d(initial pos, initial vel) and
// dL/d(xsph_c).  Each checkpoint segment is replayed once, recording every
// step's intermediates (the fused step's own launchers writing into record
// buffers: predictions of every solver iteration, lambdas, the solved
// prediction, the velocity before XSPH, the sorted keys, permutation and
// lower-bound table), then the steps are differentiated in reverse.
//
// The derivative is that of the step as written (sim/integrate.cu,
// sim/pbf_lambda.cu, sim/pbf_delta_apply.cu, sim/xsph.cu, sim/boundary.cu),
// with neighbour sets held fixed within a step: a pair contributes where the
// forward found it within h (lambda: among the first maxNeighbors in walk
// order).  Clamps contribute the derivative of the branch taken: a clamped
// position axis, a clamped lambda, a lambda zeroed for too few neighbours and
// an s_corr held at its floor pass no gradient; the displacement clamp passes
// the Jacobian of d * maxDisp / |d|.  A pair's terms are symmetric (a_ji =
// -a_ij, the same weights and Jacobian), so every particle gathers both the
// terms of its own equation and those its neighbours' equations hold for it,
// from small per-particle arrays (the clamp-projected gradient of delta, the
// coefficients of lambda and the slot of each particle's last counted
// neighbour): no atomics, and the gradients are the same bits run to run.
// (With the XSPH gate on, each particle's XSPH weight depends on its
// neighbour count; that case scatters with float atomics.)
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/pbf/pbf.h"
#include "../../include/pbf/simulator.h"
#include "fused.cuh"
#include "handle.h"
#include "grid.cuh"
#include "pbf_common.cuh"
#include "sort.cuh"

namespace pbf {
namespace {

constexpr int kBS = 256;
constexpr int kAdjBS = 128;

__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ void atomic_add3(float4* p, float3 v) {
    atomicAdd(&p->x, v.x);
    atomicAdd(&p->y, v.y);
    atomicAdd(&p->z, v.z);
}
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Pair geometry of (i, j) as the forward computes it: u = x_i - x_j, r2, and
// the spiky gradient a = coeff(r) u with its Jacobian applied to a vector.
struct Pair {
    float3 u;
    float r2, r, coeff, dcoeff;  // dcoeff = d coeff / d r
};

__device__ __forceinline__ Pair pair_of(float4 xi, float4 xj, const sim::DeviceParams& dp) {
    Pair q;
    float rx, ry, rz;
    q.r2 = dist2(xi, xj, rx, ry, rz);
    q.u = make_float3(rx, ry, rz);
    q.r = sqrt_(q.r2);
    const float h = dp.kernel.h, s = dp.kernel.spiky, eps = dp.pbf.grad_r_eps;
    const float t = h - q.r;
    const float rs = fmaxf(q.r, eps);
    q.coeff = div_(mul_(mul_(-3.0f, s), mul_(t, t)), rs);
    // coeff(r) = -3 s (h - r)^2 / max(r, eps)
    q.dcoeff = (q.r > eps) ? 3.0f * s * t * (h + q.r) / (q.r * q.r) : 6.0f * s * t / eps;
    return q;
}

// J^T g for J = d a / d u = coeff I + (coeff'/r) u u^T.
__device__ __forceinline__ float3 jt(const Pair& q, float3 g) {
    const float k = (q.r > 0.f) ? q.dcoeff / q.r * dot3(q.u, g) : 0.f;
    return make_float3(q.coeff * g.x + k * q.u.x, q.coeff * g.y + k * q.u.y, q.coeff * g.z + k * q.u.z);
}

// The neighbour candidates of a recorded step: the step's neighbour list
// (32-bit slots, walk order, built at the step's prediction with a radius
// covering all its passes) or, where a list overflowed or none was kept, the
// stencil rows of the start-of-step cell.
struct Cand {
    const uint32_t* __restrict__ key_s;
    const uint32_t* __restrict__ lb;
    const uint32_t* __restrict__ list;   // may be null
    const uint32_t* __restrict__ count;
    uint32_t cap;
};

template <class Visit>
__device__ __forceinline__ void for_candidates(uint32_t s, const Cand& c, const sim::DeviceParams& dp,
                                               Visit&& visit) {
    if (c.list) {
        const uint32_t n = c.count[s];
        if (n <= c.cap) {
            const uint32_t* l = c.list + size_t(s) * c.cap;
            for (uint32_t e = 0; e < n; ++e)
                if (!visit(__ldg(l + e))) return;
            return;
        }
    }
    int cx, cy, cz;
    decode_key(c.key_s[s], dp.grid.dim, cx, cy, cz);
    walk_neighbours(cx, cy, cz, neighbour_reach(dp), dp.grid.dim, LbRows{c.lb}, visit);
}

// The same candidates with the forward passes' queued warp walk: each lane
// queues its hits (hit(k), the cheap test) in a shared-memory ring and the
// warp runs the bodies in bulk, each lane in its own walk order.  A warp walks
// the stencil rows when any of its lists overflowed or none was kept.  Every
// lane of the warp calls it; q is the lane's queue (kAdjQ entries, stride
// kAdjBS).
constexpr int kAdjQ = 32;
template <class Hit, class Body>
__device__ __forceinline__ void adj_walk(bool active, uint32_t s, const Cand& c, const sim::DeviceParams& dp,
                                         uint32_t* q, Hit&& hit, Body&& body) {
    uint32_t n = 0;
    bool lists = c.list != nullptr;
    if (lists) {
        n = active ? c.count[s] : 0u;
        lists = !__any_sync(0xFFFFFFFFu, n > c.cap);
    }
    if (lists) {
        walk_list_queued<kAdjQ, kAdjBS, false>(active, ListSource<uint32_t>{c.list + size_t(s) * c.cap, n, s}, q,
                                        0x7FFFFFFF, hit, body);
    } else {
        int cx, cy, cz;
        decode_key(c.key_s[s], dp.grid.dim, cx, cy, cz);
        walk_queued<kAdjQ, kAdjBS, false>(active, cx, cy, cz, neighbour_reach(dp), dp.grid.dim, LbRows{c.lb}, q,
                                   0x7FFFFFFF, hit, body);
    }
}

// ---------------------------------------------------------------- XSPH
// v''_i = v_i + c g (m / rho0) sum_j (v_j - v_i) W_ij at the solved positions.
__global__ void __launch_bounds__(kAdjBS) k_adj_xsph(const float4* __restrict__ xf, const float4* __restrict__ vf,
                                                     Cand cand, const sim::DeviceParams* __restrict__ dpp,
                                                     uint32_t N, const float4* __restrict__ vbar_out,
                                                     float4* __restrict__ vfbar, float4* __restrict__ xfbar,
                                                     float* __restrict__ cbar) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    float cpart = 0.f;
    if (s < N) {
        const sim::DeviceParams& dp = *dpp;
        const float4 xi = xf[s], vi = vf[s];
        const float3 g = f3(vbar_out[s]);
        float gate = 1.0f;
        if (dp.pbf.xsph_gate_enable) {  // the gate counts neighbours first
            int count = 0;
            for_candidates(s, cand, dp, [&](uint32_t k) -> bool {
                float rx, ry, rz;
                if (k != s && !(dist2(xi, xf[k], rx, ry, rz) > dp.kernel.h2)) ++count;
                return true;
            });
            const int nMin = max(0, dp.pbf.xsph_n_min);
            const int nMax = max(nMin + 1, dp.pbf.xsph_n_max);
            gate = fminf(1.f, fmaxf(0.f, (float(count) - float(nMin)) / float(nMax - nMin)));
        }
        const float mor = (dp.restDensity > 0.f) ? dp.particleMass / dp.restDensity : 0.f;
        const float ceff = dp.xsph_c * gate * mor;
        float wsum = 0.f;
        float3 sum = make_float3(0.f, 0.f, 0.f);
        float3 own = make_float3(0.f, 0.f, 0.f);
        for_candidates(s, cand, dp, [&](uint32_t k) -> bool {
            if (k == s) return true;
            float rx, ry, rz;
            const float r2 = dist2(xi, xf[k], rx, ry, rz);
            if (r2 > dp.kernel.h2) return true;
            const float hr2 = sub_(dp.kernel.h2, r2);
            const float w = mul_(mul_(mul_(dp.kernel.poly6, hr2), hr2), hr2);
            const float4 vj = vf[k];
            const float3 dv = make_float3(vj.x - vi.x, vj.y - vi.y, vj.z - vi.z);
            sum.x += dv.x * w;
            sum.y += dv.y * w;
            sum.z += dv.z * w;
            wsum += w;
            atomic_add3(vfbar + k, make_float3(ceff * w * g.x, ceff * w * g.y, ceff * w * g.z));
            const float r2bar = ceff * dot3(dv, g) * (-3.0f * dp.kernel.poly6 * hr2 * hr2);
            const float3 ub = make_float3(2.f * rx * r2bar, 2.f * ry * r2bar, 2.f * rz * r2bar);
            own.x += ub.x;
            own.y += ub.y;
            own.z += ub.z;
            atomic_add3(xfbar + k, make_float3(-ub.x, -ub.y, -ub.z));
            return true;
        });
        cpart = gate * mor * dot3(sum, g);
        atomic_add3(vfbar + s, make_float3(g.x - ceff * wsum * g.x, g.y - ceff * wsum * g.y, g.z - ceff * wsum * g.z));
        atomic_add3(xfbar + s, own);
    }
    // dL/dc: block sum, one atomic per block
    __shared__ float red[kAdjBS];
    red[threadIdx.x] = cpart;
    __syncthreads();
    for (int w = kAdjBS / 2; w > 0; w >>= 1) {
        if (int(threadIdx.x) < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0 && cbar) atomicAdd(cbar, red[0]);
}

// Gathered XSPH adjoint (gate off: the weight c (m / rho0) is the same for
// every particle).  Particle j collects
//   dL/dv_j = g_j (1 - c sum_k W_jk) + c sum_k W_jk g_k,
//   dL/dx_j += sum_k 2 (x_j - x_k) c W'(r2) (v_k - v_j) . (g_j - g_k),
// with W'(r2) = -3 poly6 (h^2 - r2)^2, and its part of dL/dc in a per-block
// partial (summed in a fixed order by k_sum_partials).
__global__ void __launch_bounds__(kAdjBS, 6) k_adj_xsph_gather(const float4* __restrict__ xf,
                                                            const float4* __restrict__ vf, Cand cand,
                                                            const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                            const float4* __restrict__ vbar_out,
                                                            float4* __restrict__ vfbar, float4* __restrict__ xfbar,
                                                            float* __restrict__ cpart_blocks) {
    __shared__ uint32_t qs[kAdjQ * kAdjBS];
    const uint32_t s0 = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = s0 < N;  // every lane takes part in the warp-wide walk
    const uint32_t s = active ? s0 : 0u;
    const sim::DeviceParams dp = *dpp;
    const float4 xi = xf[s], vi = vf[s];
    const float3 g = f3(vbar_out[s]);
    const float mor = (dp.restDensity > 0.f) ? dp.particleMass / dp.restDensity : 0.f;
    const float ceff = dp.xsph_c * mor;
    float wsum = 0.f;
    float3 sum = make_float3(0.f, 0.f, 0.f), gsum = make_float3(0.f, 0.f, 0.f), xb = make_float3(0.f, 0.f, 0.f);
    adj_walk(
        active, s, cand, dp, qs + threadIdx.x,
        [&](uint32_t k) -> bool {
            float rx, ry, rz;
            return k != s && !(dist2(xi, xf[k], rx, ry, rz) > dp.kernel.h2);
        },
        [&](uint32_t k) {
            float rx, ry, rz;
            const float r2 = dist2(xi, xf[k], rx, ry, rz);
            const float hr2 = sub_(dp.kernel.h2, r2);
            const float w = mul_(mul_(mul_(dp.kernel.poly6, hr2), hr2), hr2);
            const float4 vj = vf[k];
            const float3 gk = f3(vbar_out[k]);
            const float3 dv = make_float3(vj.x - vi.x, vj.y - vi.y, vj.z - vi.z);
            sum.x += dv.x * w;
            sum.y += dv.y * w;
            sum.z += dv.z * w;
            wsum += w;
            gsum.x += gk.x * w;
            gsum.y += gk.y * w;
            gsum.z += gk.z * w;
            const float3 dg = make_float3(g.x - gk.x, g.y - gk.y, g.z - gk.z);
            const float r2bar = ceff * dot3(dv, dg) * (-3.0f * dp.kernel.poly6 * hr2 * hr2);
            xb.x += 2.f * rx * r2bar;
            xb.y += 2.f * ry * r2bar;
            xb.z += 2.f * rz * r2bar;
        });
    float cpart = 0.f;
    if (active) {
        cpart = mor * dot3(sum, g);
        vfbar[s] = make_float4(g.x - ceff * wsum * g.x + ceff * gsum.x, g.y - ceff * wsum * g.y + ceff * gsum.y,
                               g.z - ceff * wsum * g.z + ceff * gsum.z, 0.f);
        const float4 x0 = xfbar[s];
        xfbar[s] = make_float4(x0.x + xb.x, x0.y + xb.y, x0.z + xb.z, 0.f);
    }
    __shared__ float red[kAdjBS];
    red[threadIdx.x] = cpart;
    __syncthreads();
    for (int w = kAdjBS / 2; w > 0; w >>= 1) {
        if (int(threadIdx.x) < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) cpart_blocks[blockIdx.x] = red[0];
}

// *out += the sum of n partials, in a fixed order (one block).
__global__ void __launch_bounds__(256) k_sum_partials(const float* __restrict__ part, uint32_t n,
                                                      float* __restrict__ out) {
    __shared__ float red[256];
    float v = 0.f;
    for (uint32_t i = threadIdx.x; i < n; i += 256) v += part[i];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (int(threadIdx.x) < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out += red[0];
}

// v_f = (x_f - p) / dt; x_f = clamp(x_iters).  Writes dL/dx_iters and
// dL/dp (sorted).
__global__ void __launch_bounds__(kBS) k_adj_velocity(const float4* __restrict__ xf,
                                                      const float4* __restrict__ vfbar,
                                                      const float4* __restrict__ xfbar,
                                                      const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                      float4* __restrict__ xbar, float4* __restrict__ pbar_s,
                                                      int iters) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const sim::DeviceParams& dp = *dpp;
    const float inv_dt = 1.0f / dp.dt;
    const float4 vb = vfbar[s], xb = xfbar[s], x = xf[s];
    float3 g = make_float3(xb.x + vb.x * inv_dt, xb.y + vb.y * inv_dt, xb.z + vb.z * inv_dt);
    pbar_s[s] = make_float4(-vb.x * inv_dt, -vb.y * inv_dt, -vb.z * inv_dt, 0.f);
    // the post-solve clamp (only when iterations ran; otherwise x_f is the
    // prediction, whose own clamp the predict adjoint applies)
    if (iters > 0) {
        const sim::GridBounds& gb = dp.grid;
        if (x.x <= gb.mins.x || x.x >= gb.maxs.x) g.x = 0.f;
        if (x.y <= gb.mins.y || x.y >= gb.maxs.y) g.y = 0.f;
        if (x.z <= gb.mins.z || x.z >= gb.maxs.z) g.z = 0.f;
    }
    xbar[s] = make_float4(g.x, g.y, g.z, 0.f);
}

// ----------------------------------------------------------------- delta
// x^{k+1}_i = x^k_i + clampDisp(relax / rho0 * sum_j (l_i + l_j + scorr_ij) a_ij)
// First, per particle: Db_i = (relax / rho0) J_clamp^T dL/dx^{k+1}_i, J_clamp
// the Jacobian of the displacement clamp at the recorded pre-clamp sum.
__global__ void __launch_bounds__(kBS) k_adj_delta_db(const float4* __restrict__ dsum,
                                                      const float4* __restrict__ xbar_in,
                                                      const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                      float4* __restrict__ Db) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const sim::DeviceParams& dp = *dpp;
    const sim::PbfTuning& pbf = dp.pbf;
    const float3 D = f3(dsum[s]);
    const float3 gin = f3(xbar_in[s]);
    const float invRest = (dp.restDensity > 0.f) ? 1.0f / dp.restDensity : 0.f;
    const float omega = pbf.enable_relax ? pbf.relax_omega : 1.0f;
    const float3 d = make_float3(D.x * invRest * omega, D.y * invRest * omega, D.z * invRest * omega);
    float3 db = gin;
    if (pbf.enable_disp_clamp) {
        const float md = pbf.disp_clamp_max_h * dp.kernel.h;
        const float L2 = dot3(d, d);
        if (L2 > md * md) {
            const float L = sqrtf(L2);
            const float sc = md / (L + 1e-20f);
            const float proj = dot3(d, gin) / L2;
            db = make_float3(sc * (gin.x - d.x * proj), sc * (gin.y - d.y * proj), sc * (gin.z - d.z * proj));
        }
    }
    Db[s] = make_float4(db.x * invRest * omega, db.y * invRest * omega, db.z * invRest * omega, 0.f);
}

// Then each particle j gathers over its neighbours k, with dDb = Db_j - Db_k:
//   dL/dl_j = sum_k dDb . a_jk,
//   dL/dx^k_j = dL/dx^{k+1}_j + sum_k [J_jk^T (l_jk dDb) + 2 u_jk (dDb . a_jk) dscorr/dr2],
// both equations' terms of the pair at once (a_kj = -a_jk, the same l, s_corr
// and Jacobian).
__global__ void __launch_bounds__(kAdjBS, 6) k_adj_delta_gather(const float4* __restrict__ x,
                                                             const float* __restrict__ lam,
                                                             const float4* __restrict__ Db, Cand cand,
                                                             const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                             const float4* __restrict__ xbar_in,
                                                             float4* __restrict__ xbar_out,
                                                             float* __restrict__ lambar) {
    __shared__ uint32_t qs[kAdjQ * kAdjBS];
    const uint32_t s0 = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = s0 < N;  // every lane takes part in the warp-wide walk
    const uint32_t s = active ? s0 : 0u;
    const sim::DeviceParams dp = *dpp;
    const sim::PbfTuning& pbf = dp.pbf;
    const float4 xi = x[s];
    const float li = lam[s];
    const float w_q = scorr_wq(dp);
    const float3 Dbi = f3(Db[s]);
    float lown = 0.f;
    float3 own = f3(xbar_in[s]);  // identity path x^k -> x^{k+1}
    const float kcorr = pbf.scorr_k, ncorr = pbf.scorr_n;
    adj_walk(
        active, s, cand, dp, qs + threadIdx.x,
        [&](uint32_t k) -> bool {
            float rx, ry, rz;
            return k != s && !(dist2(xi, x[k], rx, ry, rz) > dp.kernel.h2);
        },
        [&](uint32_t k) {
            const Pair q = pair_of(xi, x[k], dp);
            const float3 a = make_float3(q.coeff * q.u.x, q.coeff * q.u.y, q.coeff * q.u.z);
            float scorr = 0.f, dscorr = 0.f;  // d scorr / d r2
            if (pbf.scorr_enable) {
                const float hr2 = dp.kernel.h2 - q.r2;
                const float w = dp.kernel.poly6 * hr2 * hr2 * hr2;
                const float ratio = (w_q > 0.f) ? w / w_q : 0.f;
                // ratio^n and ratio^(n-1); products for the default n = 4 (the
                // adjoint is FP32 calculus, not a replay of the forward's bits)
                float rn, rn1;
                if (ncorr == 4.0f) {
                    const float q2 = ratio * ratio;
                    rn1 = q2 * ratio;
                    rn = q2 * q2;
                } else {
                    rn = powf(ratio, ncorr);
                    rn1 = powf(ratio, ncorr - 1.0f);
                }
                scorr = -kcorr * rn;
                const bool floored = pbf.scorr_min < 0.f && scorr < pbf.scorr_min;
                if (floored) scorr = pbf.scorr_min;
                if (!floored && w_q > 0.f && ratio > 0.f)
                    dscorr = -kcorr * ncorr * rn1 * (-3.0f * dp.kernel.poly6 * hr2 * hr2) / w_q;
            }
            const float lij = li + lam[k] + scorr;
            const float3 Dbk = f3(Db[k]);
            const float3 dDb = make_float3(Dbi.x - Dbk.x, Dbi.y - Dbk.y, Dbi.z - Dbk.z);
            const float lbar = dot3(dDb, a);
            lown += lbar;
            const float3 ub = jt(q, make_float3(lij * dDb.x, lij * dDb.y, lij * dDb.z));
            const float r2bar = lbar * dscorr;
            own.x += ub.x + 2.f * q.u.x * r2bar;
            own.y += ub.y + 2.f * q.u.y * r2bar;
            own.z += ub.z + 2.f * q.u.z * r2bar;
        });
    if (!active) return;
    lambar[s] = lown;
    xbar_out[s] = make_float4(own.x, own.y, own.z, 0.f);
}

// ---------------------------------------------------------------- lambda
// lambda_i = -(rho_i / rho0 - 1) / (scale^2 (sum_j |a_ij|^2 + |sum_j a_ij|^2) + eps)
// First, per particle, from the recorded neighbour sums and dL/dlambda_i: the
// coefficients of its pair terms, c0 = (G, sb), c1 = (rhob, bits of the slot
// of its last counted neighbour), zero where the forward's branches pass no
// gradient (lambda zeroed, not finite or clamped).
__global__ void __launch_bounds__(kBS) k_adj_lambda_coef(const float4* __restrict__ accs,
                                                         const float* __restrict__ lambar,
                                                         const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                         float4* __restrict__ coef) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const sim::DeviceParams& dp = *dpp;
    const sim::PbfTuning& pbf = dp.pbf;
    const float4 a0 = accs[2 * size_t(s)], a1 = accs[2 * size_t(s) + 1];
    float4 c0 = make_float4(0.f, 0.f, 0.f, 0.f), c1 = make_float4(0.f, a1.z, 0.f, 0.f);
    const float lb_i = lambar[s];
    const float rho0 = dp.restDensity;
    const float scale = (rho0 > 0.f) ? dp.particleMass / rho0 : 0.f;
    const float gx = a0.z, gy = a0.w, gz = a1.x;
    const float G2 = gx * gx + gy * gy + gz * gz;
    const float sum = a0.y + G2;
    float denom0 = scale * scale * sum + pbf.lambda_denom_eps;
    if (pbf.compliance > 0.f && dp.dt > 0.f) denom0 += pbf.compliance / (dp.dt * dp.dt);
    const float denom = fmaxf(denom0, pbf.lambda_denom_eps);
    const int contrib = int(a1.y);
    bool live = lb_i != 0.f && !(contrib < 2 || sum < 1e-12f || !(rho0 > 0.f));
    float lam = 0.f;
    if (live) {
        lam = -(a0.x / rho0 - 1.f) / denom;
        live = isfinite(lam) && !(pbf.enable_lambda_clamp && fabsf(lam) > pbf.lambda_max_abs);
    }
    if (live) {
        const float Cb = -lb_i / denom;
        const float denb = (denom0 >= pbf.lambda_denom_eps) ? -lb_i * lam / denom : 0.f;
        c0 = make_float4(gx, gy, gz, denb * scale * scale);
        c1.x = Cb / rho0;
    }
    coef[2 * size_t(s)] = c0;
    coef[2 * size_t(s) + 1] = c1;
}

// Then each particle j gathers, over its neighbours k in walk order, the term
// of its own equation (for its first maxNeighbors neighbours) and the term of
// k's equation when j was among k's counted neighbours (walks visit slots in
// ascending order, so: slot j <= k's last counted slot):
//   dL/dx_j += J_jk^T (2 sb_j (a_jk + G_j)) + 2 u_jk rhob_j m W'(r2)
//            - J_jk^T (2 sb_k (G_k - a_jk)) + 2 u_jk rhob_k m W'(r2).
__global__ void __launch_bounds__(kAdjBS, 6) k_adj_lambda_gather(const float4* __restrict__ x,
                                                              const float4* __restrict__ coef, Cand cand,
                                                              const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                              float4* __restrict__ xbar_out) {
    __shared__ uint32_t qs[kAdjQ * kAdjBS];
    const uint32_t s0 = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = s0 < N;  // every lane takes part in the warp-wide walk
    const uint32_t s = active ? s0 : 0u;
    const sim::DeviceParams dp = *dpp;
    const float4 xi = x[s];
    const int cap = dp.maxNeighbors > 0 ? dp.maxNeighbors : 0x7FFFFFFF;
    const float4 ci0 = coef[2 * size_t(s)], ci1 = coef[2 * size_t(s) + 1];
    const float3 Gi = f3(ci0);
    const float sbi = ci0.w, rhobi = ci1.x;
    const bool liveI = sbi != 0.f || rhobi != 0.f;
    const float mp6 = -3.0f * dp.particleMass * dp.kernel.poly6;
    float3 acc = make_float3(0.f, 0.f, 0.f);
    int seen = 0;
    adj_walk(
        active, s, cand, dp, qs + threadIdx.x,
        [&](uint32_t k) -> bool {
            float rx, ry, rz;
            return k != s && !(dist2(xi, x[k], rx, ry, rz) > dp.kernel.h2);
        },
        [&](uint32_t k) {
            const Pair q = pair_of(xi, x[k], dp);
            const float3 a = make_float3(q.coeff * q.u.x, q.coeff * q.u.y, q.coeff * q.u.z);
            const float hr2 = dp.kernel.h2 - q.r2;
            const float dW = mp6 * hr2 * hr2;
            if (seen < cap && liveI) {
                const float3 ub = jt(q, make_float3(2.f * sbi * (a.x + Gi.x), 2.f * sbi * (a.y + Gi.y),
                                                    2.f * sbi * (a.z + Gi.z)));
                const float r2bar = rhobi * dW;
                acc.x += ub.x + 2.f * q.u.x * r2bar;
                acc.y += ub.y + 2.f * q.u.y * r2bar;
                acc.z += ub.z + 2.f * q.u.z * r2bar;
            }
            ++seen;
            const float4 ck0 = coef[2 * size_t(k)], ck1 = coef[2 * size_t(k) + 1];
            if (s <= __float_as_uint(ck1.y) && (ck0.w != 0.f || ck1.x != 0.f)) {
                const float sbk = ck0.w;
                const float3 ub = jt(q, make_float3(2.f * sbk * (ck0.x - a.x), 2.f * sbk * (ck0.y - a.y),
                                                    2.f * sbk * (ck0.z - a.z)));
                const float r2bar = ck1.x * dW;
                acc.x += -ub.x + 2.f * q.u.x * r2bar;
                acc.y += -ub.y + 2.f * q.u.y * r2bar;
                acc.z += -ub.z + 2.f * q.u.z * r2bar;
            }
        });
    if (!active) return;
    const float4 o = xbar_out[s];
    xbar_out[s] = make_float4(o.x + acc.x, o.y + acc.y, o.z + acc.z, 0.f);
}

// ---------------------------------------------------------------- predict
// x^0 = clamp(p + (v + g dt) dt); scatter dL/dp and dL/dv to particle ids.
__global__ void __launch_bounds__(kBS) k_adj_predict(const float4* __restrict__ x0,
                                                     const float4* __restrict__ xbar0,
                                                     const float4* __restrict__ pbar_s,
                                                     const uint32_t* __restrict__ perm,
                                                     const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                     float4* __restrict__ pbar, float4* __restrict__ vbar) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const sim::DeviceParams& dp = *dpp;
    const sim::GridBounds& gb = dp.grid;
    const float4 x = x0[s];
    float3 g = f3(xbar0[s]);
    if (x.x <= gb.mins.x || x.x >= gb.maxs.x) g.x = 0.f;
    if (x.y <= gb.mins.y || x.y >= gb.maxs.y) g.y = 0.f;
    if (x.z <= gb.mins.z || x.z >= gb.maxs.z) g.z = 0.f;
    const float4 pb = pbar_s[s];
    const uint32_t i = perm[s];
    pbar[i] = make_float4(pb.x + g.x, pb.y + g.y, pb.z + g.z, 0.f);
    vbar[i] = make_float4(dp.dt * g.x, dp.dt * g.y, dp.dt * g.z, 0.f);
}

// dL/d(outputs) of a step in sorted order: x_f[s] is p_{n+1}[perm[s]].
__global__ void __launch_bounds__(kBS) k_adj_gather_out(const uint32_t* __restrict__ perm,
                                                        const float4* __restrict__ pbar,
                                                        const float4* __restrict__ vbar, uint32_t N,
                                                        float4* __restrict__ xfbar, float4* __restrict__ vxbar) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const uint32_t i = perm[s];
    xfbar[s] = pbar[i];
    vxbar[s] = vbar[i];
}

// --------------------------------------------------------- grid density loss
// rho(g) = sum_i m W(|g - p_i|) on res^3 cell centres of the box.
struct GridDesc {
    float3 lo, step;
    int res;
};

__device__ __forceinline__ void grid_range(float c, float lo, float step, float h, int res, int& a, int& b) {
    a = max(0, int(ceilf((c - h - lo) / step - 0.5f)));
    b = min(res - 1, int(floorf((c + h - lo) / step - 0.5f)));
}

__global__ void __launch_bounds__(kBS) k_grid_density(const float4* __restrict__ pos,
                                                      const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                      GridDesc gd, float* __restrict__ rho) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const sim::DeviceParams& dp = *dpp;
    const float h = dp.kernel.h, h2 = dp.kernel.h2;
    const float4 p = pos[i];
    int x0, x1, y0, y1, z0, z1;
    grid_range(p.x, gd.lo.x, gd.step.x, h, gd.res, x0, x1);
    grid_range(p.y, gd.lo.y, gd.step.y, h, gd.res, y0, y1);
    grid_range(p.z, gd.lo.z, gd.step.z, h, gd.res, z0, z1);
    for (int z = z0; z <= z1; ++z)
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                const float gx = gd.lo.x + (x + 0.5f) * gd.step.x, gy = gd.lo.y + (y + 0.5f) * gd.step.y,
                            gz = gd.lo.z + (z + 0.5f) * gd.step.z;
                const float dx = gx - p.x, dy = gy - p.y, dz = gz - p.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 >= h2) continue;
                const float hr2 = h2 - r2;
                atomicAdd(rho + (size_t(z) * gd.res + y) * gd.res + x, dp.particleMass * dp.kernel.poly6 * hr2 * hr2 * hr2);
            }
}

// Residuals r = rho - target and the loss sum (one partial per block).
__global__ void __launch_bounds__(kBS) k_grid_residual(float* __restrict__ rho, const float* __restrict__ target,
                                                       uint32_t G, double* __restrict__ partial) {
    __shared__ double red[kBS];
    double acc = 0.0;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < G; g += gridDim.x * blockDim.x) {
        const float r = rho[g] - target[g];
        rho[g] = r;
        acc += double(r) * double(r);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kBS / 2; w > 0; w >>= 1) {
        if (int(threadIdx.x) < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// dL/dp_i = 2/G sum_g r_g m dW(g - p_i)/dp_i.
__global__ void __launch_bounds__(kBS) k_grid_loss_grad(const float4* __restrict__ pos,
                                                        const sim::DeviceParams* __restrict__ dpp, uint32_t N,
                                                        GridDesc gd, const float* __restrict__ resid,
                                                        float scale, float4* __restrict__ pbar) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const sim::DeviceParams& dp = *dpp;
    const float h = dp.kernel.h, h2 = dp.kernel.h2;
    const float4 p = pos[i];
    int x0, x1, y0, y1, z0, z1;
    grid_range(p.x, gd.lo.x, gd.step.x, h, gd.res, x0, x1);
    grid_range(p.y, gd.lo.y, gd.step.y, h, gd.res, y0, y1);
    grid_range(p.z, gd.lo.z, gd.step.z, h, gd.res, z0, z1);
    float3 g = make_float3(0.f, 0.f, 0.f);
    for (int z = z0; z <= z1; ++z)
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                const float gx = gd.lo.x + (x + 0.5f) * gd.step.x, gy = gd.lo.y + (y + 0.5f) * gd.step.y,
                            gz = gd.lo.z + (z + 0.5f) * gd.step.z;
                const float dx = p.x - gx, dy = p.y - gy, dz = p.z - gz;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 >= h2) continue;
                const float hr2 = h2 - r2;
                // dW/dp = poly6 * 3 hr2^2 * (-2 (p - g))
                const float c = scale * resid[(size_t(z) * gd.res + y) * gd.res + x] * dp.particleMass *
                                dp.kernel.poly6 * (-6.0f) * hr2 * hr2;
                g.x += c * dx;
                g.y += c * dy;
                g.z += c * dz;
            }
    pbar[i] = make_float4(g.x, g.y, g.z, 0.f);
}

template <class T>
bool dalloc(T** p, size_t count) {
    if (count == 0) count = 1;
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * count) == cudaSuccess;
}

int status_of(cudaError_t e) {
    if (e == cudaSuccess) return PBF_OK;
    if (e == cudaErrorMemoryAllocation) return PBF_ERR_OOM;
    return PBF_ERR_CUDA;
}

GridDesc grid_desc(const sim::GridBounds& g, int res) {
    GridDesc d;
    d.res = res;
    d.lo = g.mins;
    d.step = make_float3((g.maxs.x - g.mins.x) / res, (g.maxs.y - g.mins.y) / res, (g.maxs.z - g.mins.z) / res);
    return d;
}

// One step's recorded intermediates (sorted order).
struct StepRecord {
    std::vector<float4*> x;  // x[0..iters]: predictions of each iteration; x[iters] = solved (clamped)
    std::vector<float*> lam;  // lambda of each iteration
    std::vector<float4*> D;   // delta's neighbour sum of each iteration (before the clamp)
    std::vector<float4*> A;   // lambda's neighbour sums of each iteration (2 float4 per particle)
    float4* vf = nullptr;     // velocity before XSPH
    float4* ps = nullptr;     // step-start positions
    uint32_t* key_s = nullptr;
    uint32_t* perm = nullptr;
    uint32_t* lb = nullptr;
    uint32_t* list = nullptr;   // the step's neighbour lists (null: none kept)
    uint32_t* count = nullptr;
};

}  // namespace
}  // namespace pbf

struct pbf_tape {
    sim::SimParams p{};
    uint32_t N = 0, numCells = 0;
    int steps = 0, every = 1, iters = 0, keyBits = 1;
    bool xsph = false;
    bool fast = false;  // the forward's arithmetic mode: the replay uses the same delta pass
    cudaStream_t stream = nullptr;
    // replay engine (the fused step's buffers)
    float4 *pos = nullptr, *vel = nullptr;
    float4* xl = nullptr;  // the lambda pass's (x, y, z, lambda), read by the delta pass
    uint32_t* keys = nullptr;
    sim::DeviceParams* dp = nullptr;
    uint32_t* err = nullptr;
    void* sortTemp = nullptr;
    size_t sortBytes = 0;
    // checkpoints (device): state at steps 0, every, 2 every, ...
    std::vector<float4*> ckPos, ckVel;
    std::vector<pbf::StepRecord> rec;  // one segment
    // adjoint scratch
    float4 *pbar = nullptr, *vbar = nullptr, *xfbar = nullptr, *vxbar = nullptr, *vfbar = nullptr, *xbA = nullptr,
           *xbB = nullptr, *pbar_s = nullptr;
    float *lambar = nullptr, *cbar = nullptr;
    float4* Db = nullptr;     // delta adjoint: clamp-projected gradient per particle
    float4* lcoef = nullptr;  // lambda adjoint: pair-term coefficients, 2 per particle
    float* cpart = nullptr;   // XSPH adjoint: per-block partials of dL/dc
    uint32_t* listStats = nullptr;
    uint32_t listCap = 0;  // 0: the replay walks the stencil
    int listSpan = 0;
    std::vector<void*> owned;

    template <class T>
    bool alloc(T** ptr, size_t count) {
        if (!pbf::dalloc(ptr, count)) return false;
        owned.push_back(*ptr);
        return true;
    }
    ~pbf_tape() {
        if (stream) cudaStreamSynchronize(stream);
        for (void* q : owned) cudaFree(q);
        if (stream) cudaStreamDestroy(stream);
    }

    pbf::FusedShape shape() const {
        pbf::FusedShape sh{};
        sh.N = N;
        sh.numCells = numCells;
        sh.key_bits = keyBits;
        sh.iters = iters;
        sh.hashed = false;
        sh.xsph = xsph;
        sh.list_span = listCap ? listSpan : 0;
        sh.fast = fast;
        return sh;
    }

    // Steps the replay engine once, recording into r.
    cudaError_t record_step(const pbf::StepRecord& r) {
        using namespace pbf;
        const FusedShape sh = shape();
        FusedBufs b{};
        b.pos = pos;
        b.vel = vel;
        b.keys = keys;
        b.key_s = r.key_s;
        b.perm = r.perm;
        b.pred_a = r.x[0];
        b.pred_b = xl;
        b.pos_s = r.ps;
        b.vel_s = r.vf;
        b.lam_s = r.lam.empty() ? nullptr : r.lam[0];
        b.lb = r.lb;
        b.sort_temp = sortTemp;
        b.sort_bytes = sortBytes;
        b.dp = dp;
        b.err = err;
        b.nbr_list = r.list;
        b.nbr_count = r.count;
        b.nbr_stats = listStats;
        b.nbr_cap = r.list ? listCap : 0u;
        b.nbr_staging = false;
        cudaError_t e;
        if ((e = fused_predict_keys(b, sh, stream)) != cudaSuccess) return e;
        if ((e = fused_sort(b, sh, stream)) != cudaSuccess) return e;
        if ((e = fused_gather_and_tables(b, sh, stream)) != cudaSuccess) return e;
        e = fused_build_lists(b, sh, 0, stream);
        if (e != cudaSuccess && e != cudaErrorNotReady) return e;
        if (iters <= 0) {
            if ((e = fused_solve(b, sh, stream)) != cudaSuccess) return e;  // boundary + velocity on x[0]
        }
        for (int it = 0; it < iters; ++it) {
            FusedBufs bi = b;
            bi.pred_a = r.x[it];
            bi.pred_next = r.x[it + 1];
            bi.lam_s = r.lam[it];
            bi.delta_sum = r.D[it];
            bi.lambda_acc = r.A[it];
            if ((e = fused_solve_phase(bi, sh, it, 0, stream)) != cudaSuccess) return e;
            if ((e = fused_solve_phase(bi, sh, it, 1, stream)) != cudaSuccess) return e;
        }
        FusedBufs bc = b;
        bc.pred_a = r.x[std::max(iters, 0)];
        return fused_commit(bc, sh, stream);
    }

    // dL/d(outputs of the recorded step) in pbar/vbar (ids) -> dL/d(inputs).
    cudaError_t adjoint_step(const pbf::StepRecord& r) {
        using namespace pbf;
        const unsigned g = blocks_for(N, kBS), ga = blocks_for(N, kAdjBS);
        const size_t b4 = sizeof(float4) * N;
        k_adj_gather_out<<<g, kBS, 0, stream>>>(r.perm, pbar, vbar, N, xfbar, vxbar);
        const float4* xf = r.x[std::max(iters, 0)];
        const Cand cand{r.key_s, r.lb, r.list, r.count, listCap};
        if (xsph && p.pbf.xsph_gate_enable) {
            cudaMemsetAsync(vfbar, 0, b4, stream);
            k_adj_xsph<<<ga, kAdjBS, 0, stream>>>(xf, r.vf, cand, dp, N, vxbar, vfbar, xfbar, cbar);
        } else if (xsph) {
            k_adj_xsph_gather<<<ga, kAdjBS, 0, stream>>>(xf, r.vf, cand, dp, N, vxbar, vfbar, xfbar, cpart);
            k_sum_partials<<<1, 256, 0, stream>>>(cpart, ga, cbar);
        } else {
            cudaMemcpyAsync(vfbar, vxbar, b4, cudaMemcpyDeviceToDevice, stream);
        }
        k_adj_velocity<<<g, kBS, 0, stream>>>(xf, vfbar, xfbar, dp, N, xbA, pbar_s, iters);
        float4* xin = xbA;
        float4* xout = xbB;
        for (int it = iters - 1; it >= 0; --it) {
            k_adj_delta_db<<<g, kBS, 0, stream>>>(r.D[it], xin, dp, N, Db);
            k_adj_delta_gather<<<ga, kAdjBS, 0, stream>>>(r.x[it], r.lam[it], Db, cand, dp, N, xin, xout, lambar);
            k_adj_lambda_coef<<<g, kBS, 0, stream>>>(r.A[it], lambar, dp, N, lcoef);
            k_adj_lambda_gather<<<ga, kAdjBS, 0, stream>>>(r.x[it], lcoef, cand, dp, N, xout);
            std::swap(xin, xout);
        }
        k_adj_predict<<<g, kBS, 0, stream>>>(r.x[0], xin, pbar_s, r.perm, dp, N, pbar, vbar);
        return cudaGetLastError();
    }
};

namespace {

int make_tape(const sim::SimParams& sp, uint32_t N, int steps, int every, bool xsph, pbf_tape** out) {
    using namespace pbf;
    pbf_tape* t = new (std::nothrow) pbf_tape;
    if (!t) return PBF_ERR_OOM;
    t->p = sp;
    t->N = N;
    t->steps = steps;
    t->every = every;
    t->iters = sp.solverIters;
    t->xsph = xsph;
    const int3 d = sp.grid.dim;
    t->numCells = uint32_t(d.x) * uint32_t(d.y) * uint32_t(d.z);
    t->keyBits = bits_for(t->numCells - 1u);
    t->sortBytes = sort_temp_bytes(N, t->keyBits);
    const int segs = (steps + every - 1) / every;
    // Keep each recorded step's neighbour lists when one list serves the
    // whole step (the single-list schedule) and they fit in a quarter of the
    // free device memory.
    const int span = list_span_for(sp);
    if (span >= sp.solverIters && span > 0) {
        size_t freeB = 0, totalB = 0;
        cudaMemGetInfo(&freeB, &totalB);
        const uint32_t cap = sim::Simulator::kDefaultListCapacity;
        const size_t need = size_t(std::min(every, steps)) * N * (size_t(cap) + 1) * sizeof(uint32_t);
        if (need <= freeB / 4) {
            t->listCap = cap;
            t->listSpan = span;
        }
    }
    bool ok = cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) == cudaSuccess && t->alloc(&t->pos, N) &&
              t->alloc(&t->vel, N) && t->alloc(&t->xl, N) && t->alloc(&t->keys, N) && t->alloc(&t->dp, 1) && t->alloc(&t->err, 1) &&
              t->alloc(reinterpret_cast<unsigned char**>(&t->sortTemp), t->sortBytes) && t->alloc(&t->pbar, N) &&
              t->alloc(&t->vbar, N) && t->alloc(&t->xfbar, N) && t->alloc(&t->vxbar, N) && t->alloc(&t->vfbar, N) &&
              t->alloc(&t->xbA, N) && t->alloc(&t->xbB, N) && t->alloc(&t->pbar_s, N) && t->alloc(&t->lambar, N) &&
              t->alloc(&t->Db, N) && t->alloc(&t->lcoef, 2 * size_t(N)) &&
              t->alloc(&t->cpart, size_t(blocks_for(N, kAdjBS))) &&
              t->alloc(&t->cbar, 1) && t->alloc(&t->listStats, 2);
    for (int c = 0; ok && c < segs; ++c) {
        float4 *cp = nullptr, *cv = nullptr;
        ok = t->alloc(&cp, N) && t->alloc(&cv, N);
        t->ckPos.push_back(cp);
        t->ckVel.push_back(cv);
    }
    t->rec.resize(size_t(std::min(every, steps)));
    for (auto& r : t->rec) {
        if (!ok) break;
        r.x.assign(size_t(std::max(t->iters, 0) + 1), nullptr);
        r.lam.assign(size_t(std::max(t->iters, 0)), nullptr);
        r.D.assign(size_t(std::max(t->iters, 0)), nullptr);
        r.A.assign(size_t(std::max(t->iters, 0)), nullptr);
        for (auto& x : r.x) ok = ok && t->alloc(&x, N);
        for (auto& l : r.lam) ok = ok && t->alloc(&l, N);
        for (auto& dd : r.D) ok = ok && t->alloc(&dd, N);
        for (auto& aa : r.A) ok = ok && t->alloc(&aa, 2 * size_t(N));
        ok = ok && t->alloc(&r.vf, N) && t->alloc(&r.ps, N) && t->alloc(&r.key_s, N) && t->alloc(&r.perm, N) &&
             t->alloc(&r.lb, size_t(t->numCells) + 1);
        if (ok && t->listCap) ok = t->alloc(&r.list, size_t(N) * t->listCap) && t->alloc(&r.count, N);
    }
    if (ok) {
        const sim::DeviceParams dp = sim::MakeDeviceParams(sp);
        ok = cudaMemcpy(t->dp, &dp, sizeof(dp), cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemset(t->err, 0, sizeof(uint32_t)) == cudaSuccess &&
             cudaMemset(t->listStats, 0, 2 * sizeof(uint32_t)) == cudaSuccess && fused_prepare_kernels() == cudaSuccess &&
             cudaDeviceSynchronize() == cudaSuccess;  // the legacy-stream setup, before the tape's stream runs
    }
    if (!ok) {
        const cudaError_t e = cudaGetLastError();
        delete t;
        return e == cudaErrorMemoryAllocation ? PBF_ERR_OOM : PBF_ERR_CUDA;
    }
    *out = t;
    return PBF_OK;
}

// The parts of pbf_forward / pbf_backward that a batch interleaves across its
// scenes: everything is enqueued on the scene's stream (the handle's for the
// forward, the tape's own for the backward), and nothing waits until the
// caller synchronises every stream of the batch.
int tape_for(pbf_sim* h, int steps, int every, pbf_tape** out) {
    sim::Simulator& S = h->sim;
    const sim::SimParams& sp = S.params();
    if (sp.pbf.xpbd_enable) return PBF_ERR_UNSUPPORTED;
    const int st = make_tape(sp, S.activeParticleCount(), steps, every, S.buffers().xsphEnabled && sp.xsph_c > 0.f,
                             out);
    if (st == PBF_OK) (*out)->fast = S.mathMode() == 1;
    return st;
}

// Step n of the forward: the checkpoint when n starts a segment, then the step.
bool forward_step(pbf_sim* h, pbf_tape* t, int n) {
    sim::Simulator& S = h->sim;
    if (n % t->every == 0) {
        const int c = n / t->every;
        const size_t b4 = sizeof(float4) * t->N;
        cudaStream_t s = S.cudaStream();
        if (cudaMemcpyAsync(t->ckPos[c], S.devicePositions(), b4, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(t->ckVel[c], S.deviceVel(), b4, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return false;
    }
    return S.step(t->p);
}

cudaError_t backward_begin(pbf_tape* t, const float4* d_pos_bar, const float4* d_vel_bar) {
    const size_t b4 = sizeof(float4) * t->N;
    cudaMemcpyAsync(t->pbar, d_pos_bar, b4, cudaMemcpyDeviceToDevice, t->stream);
    cudaMemcpyAsync(t->vbar, d_vel_bar, b4, cudaMemcpyDeviceToDevice, t->stream);
    return cudaMemsetAsync(t->cbar, 0, sizeof(float), t->stream);
}

cudaError_t backward_load(pbf_tape* t, int c) {
    const size_t b4 = sizeof(float4) * t->N;
    cudaMemcpyAsync(t->pos, t->ckPos[c], b4, cudaMemcpyDeviceToDevice, t->stream);
    return cudaMemcpyAsync(t->vel, t->ckVel[c], b4, cudaMemcpyDeviceToDevice, t->stream);
}

cudaError_t backward_end(pbf_tape* t, float4* d_pos0_bar, float4* d_vel0_bar) {
    const size_t b4 = sizeof(float4) * t->N;
    if (d_pos0_bar) cudaMemcpyAsync(d_pos0_bar, t->pbar, b4, cudaMemcpyDeviceToDevice, t->stream);
    if (d_vel0_bar) cudaMemcpyAsync(d_vel0_bar, t->vbar, b4, cudaMemcpyDeviceToDevice, t->stream);
    return cudaGetLastError();
}

// After the tape's stream has drained: the kernels' error word and dL/dc.
int backward_result(pbf_tape* t, float* xsph_c_bar) {
    uint32_t err = 0;
    float cb = 0.f;
    if (cudaMemcpy(&err, t->err, sizeof(err), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&cb, t->cbar, sizeof(cb), cudaMemcpyDeviceToHost) != cudaSuccess)
        return PBF_ERR_CUDA;
    if (err) return (err & pbf::kErrTimeoutBits) ? PBF_ERR_TIMEOUT : PBF_ERR_CUDA;
    if (xsph_c_bar) *xsph_c_bar = cb;
    return PBF_OK;
}

template <class T>
bool distinct(const T* const* v, int count) {
    for (int i = 0; i < count; ++i)
        for (int j = 0; j < i; ++j)
            if (v[i] == v[j]) return false;
    return true;
}

}  // namespace

extern "C" {

int pbf_forward_batch(pbf_sim* const* sims, int count, int steps, int checkpoint_every, pbf_tape** tapes) {
    if (!tapes || count <= 0) return PBF_ERR_INVALID;
    for (int i = 0; i < count; ++i) tapes[i] = nullptr;
    if (!sims || steps <= 0 || checkpoint_every <= 0) return PBF_ERR_INVALID;
    for (int i = 0; i < count; ++i)
        if (!sims[i]) return PBF_ERR_INVALID;
    if (!distinct(sims, count)) return PBF_ERR_INVALID;
    int st = PBF_OK;
    for (int i = 0; i < count && st == PBF_OK; ++i) st = tape_for(sims[i], steps, checkpoint_every, &tapes[i]);
    // Step n of every scene before step n + 1 of any: the scenes' streams
    // run side by side.
    for (int n = 0; n < steps && st == PBF_OK; ++n)
        for (int i = 0; i < count && st == PBF_OK; ++i)
            if (!forward_step(sims[i], tapes[i], n)) st = PBF_ERR_CUDA;
    for (int i = 0; i < count; ++i) {
        const cudaError_t e = cudaStreamSynchronize(sims[i]->sim.cudaStream());
        if (st == PBF_OK && e != cudaSuccess) st = pbf::status_of(e);
    }
    if (st != PBF_OK)
        for (int i = 0; i < count; ++i) {
            delete tapes[i];
            tapes[i] = nullptr;
        }
    return st;
}

int pbf_forward(pbf_sim* h, int steps, int checkpoint_every, pbf_tape** out) {
    if (!out) return PBF_ERR_INVALID;
    *out = nullptr;
    if (!h) return PBF_ERR_INVALID;
    return pbf_forward_batch(&h, 1, steps, checkpoint_every, out);
}

int pbf_backward_batch(pbf_tape* const* tapes, int count, const float4* const* d_pos_bar,
                       const float4* const* d_vel_bar, float4* const* d_pos0_bar, float4* const* d_vel0_bar,
                       float* xsph_c_bar) {
    if (!tapes || count <= 0 || !d_pos_bar || !d_vel_bar) return PBF_ERR_INVALID;
    for (int i = 0; i < count; ++i)
        if (!tapes[i] || !d_pos_bar[i] || !d_vel_bar[i] || tapes[i]->steps != tapes[0]->steps ||
            tapes[i]->every != tapes[0]->every)
            return PBF_ERR_INVALID;
    if (!distinct(tapes, count)) return PBF_ERR_INVALID;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < count && e == cudaSuccess; ++i) e = backward_begin(tapes[i], d_pos_bar[i], d_vel_bar[i]);
    const pbf_tape& t0 = *tapes[0];
    for (int c = int(t0.ckPos.size()) - 1; c >= 0 && e == cudaSuccess; --c) {
        const int len = std::min(t0.every, t0.steps - c * t0.every);
        for (int i = 0; i < count && e == cudaSuccess; ++i) e = backward_load(tapes[i], c);
        for (int n = 0; n < len && e == cudaSuccess; ++n)
            for (int i = 0; i < count && e == cudaSuccess; ++i) e = tapes[i]->record_step(tapes[i]->rec[n]);
        for (int n = len - 1; n >= 0 && e == cudaSuccess; --n)
            for (int i = 0; i < count && e == cudaSuccess; ++i) e = tapes[i]->adjoint_step(tapes[i]->rec[n]);
    }
    for (int i = 0; i < count && e == cudaSuccess; ++i)
        e = backward_end(tapes[i], d_pos0_bar ? d_pos0_bar[i] : nullptr, d_vel0_bar ? d_vel0_bar[i] : nullptr);
    int st = pbf::status_of(e);
    for (int i = 0; i < count; ++i) {
        const cudaError_t se = cudaStreamSynchronize(tapes[i]->stream);
        if (st == PBF_OK && se != cudaSuccess) st = pbf::status_of(se);
    }
    for (int i = 0; i < count && st == PBF_OK; ++i) st = backward_result(tapes[i], xsph_c_bar ? xsph_c_bar + i : nullptr);
    return st;
}

int pbf_backward(pbf_tape* t, const float4* d_pos_bar, const float4* d_vel_bar, float4* d_pos0_bar,
                 float4* d_vel0_bar, float* xsph_c_bar) {
    if (!t || !d_pos_bar || !d_vel_bar) return PBF_ERR_INVALID;
    return pbf_backward_batch(&t, 1, &d_pos_bar, &d_vel_bar, &d_pos0_bar, &d_vel0_bar, xsph_c_bar);
}

int pbf_tape_destroy(pbf_tape* t) {
    delete t;
    return PBF_OK;
}

int pbf_density_grid(pbf_sim* h, int res, float* d_grid) {
    if (!h || res <= 0 || res > 1024 || !d_grid) return PBF_ERR_INVALID;
    sim::Simulator& S = h->sim;
    const uint32_t N = S.activeParticleCount();
    cudaStream_t s = S.cudaStream();
    const size_t G = size_t(res) * res * res;
    cudaMemsetAsync(d_grid, 0, sizeof(float) * G, s);
    if (N > 0)
        pbf::k_grid_density<<<pbf::blocks_for(N, pbf::kBS), pbf::kBS, 0, s>>>(
            S.devicePositions(), S.buffers().d_params, N, pbf::grid_desc(S.params().grid, res), d_grid);
    return pbf::status_of(cudaStreamSynchronize(s));
}

int pbf_density_grid_loss(pbf_sim* h, int res, const float* d_target, double* loss, float4* d_pos_bar) {
    if (!h || res <= 0 || res > 1024 || !d_target) return PBF_ERR_INVALID;
    sim::Simulator& S = h->sim;
    const uint32_t N = S.activeParticleCount();
    cudaStream_t s = S.cudaStream();
    const uint32_t G = uint32_t(res) * res * res;
    float* rho = nullptr;
    double* partial = nullptr;
    const unsigned nb = std::min<unsigned>(1024u, pbf::blocks_for(G, pbf::kBS));
    if (cudaMallocAsync(&rho, sizeof(float) * G, s) != cudaSuccess ||
        cudaMallocAsync(&partial, sizeof(double) * nb, s) != cudaSuccess)
        return PBF_ERR_OOM;
    const pbf::GridDesc gd = pbf::grid_desc(S.params().grid, res);
    cudaMemsetAsync(rho, 0, sizeof(float) * G, s);
    if (N > 0)
        pbf::k_grid_density<<<pbf::blocks_for(N, pbf::kBS), pbf::kBS, 0, s>>>(S.devicePositions(),
                                                                            S.buffers().d_params, N, gd, rho);
    pbf::k_grid_residual<<<nb, pbf::kBS, 0, s>>>(rho, d_target, G, partial);
    if (d_pos_bar && N > 0)
        pbf::k_grid_loss_grad<<<pbf::blocks_for(N, pbf::kBS), pbf::kBS, 0, s>>>(
            S.devicePositions(), S.buffers().d_params, N, gd, rho, 2.0f / float(G), d_pos_bar);
    std::vector<double> hp(nb);
    cudaMemcpyAsync(hp.data(), partial, sizeof(double) * nb, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(rho, s);
    cudaFreeAsync(partial, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return pbf::status_of(e);
    double acc = 0.0;
    for (double v : hp) acc += v;
    if (loss) *loss = acc / double(G);
    return PBF_OK;
}

}  // extern "C"
