// pbf_common.cuh - device-side building blocks shared by every PBF kernel.
//
// The arithmetic of each helper restates one reference kernel (cited per
// function) in the same operation order, so results match the reference's
// FP32 kernels to rounding.  Neighbour walks follow the reference order
// (sim/pbf_lambda.cu:49-84): dz, dy, dx over [-reach, reach], cells outside
// [0,dim) skipped, then ascending sorted position.  Because the cells
// dx = -reach..reach of one (dz,dy) row are consecutive keys, their sorted
// ranges are adjacent, so each row is walked as ONE contiguous slot range -
// the same candidates in the same order as the reference's per-cell loop.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pbf/parameters.h"
#include "pbf_errors.h"

namespace pbf {

// ---------------------------------------------------------------- errors
// Device-side error word (per sort / per handle).  Kernels never trap: a
// bounded wait that gives up ORs a bit in here and returns.
constexpr uint32_t kErrLookbackTimeout = kErrLookbackTimeoutBit;

// Bounded spin for decoupled look-back: after this many polls the waiting
// block records kErrLookbackTimeout and treats the predecessor as done.
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Status word of a decoupled look-back: 2-bit flag | 30-bit count.
constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;

// Walks back over tile statuses [tile-1, tile-2, ...] until an inclusive
// prefix is found; returns the exclusive prefix of `tile`.  Every poll loop is
// bounded by kSpinLimit.
__device__ __forceinline__ uint32_t lookback_exclusive(const uint32_t* status, uint32_t tile, uint32_t stride,
                                                       uint32_t* err, uint32_t spin_limit = kSpinLimit) {
    uint32_t excl = 0;
    int64_t k = int64_t(tile) - 1;
    while (k >= 0) {
        const uint32_t* p = status + uint64_t(k) * stride;
        uint32_t v = ld_relaxed(p);
        uint32_t spins = 0;
        while ((v & kFlagMask) == 0u) {
            if (++spins > spin_limit) {
                atomicOr(err, kErrLookbackTimeout);
                return excl;
            }
            __nanosleep(32);
            v = ld_relaxed(p);
        }
        excl += v & kCountMask;
        if ((v & kFlagMask) == kFlagPrefix) break;
        --k;
    }
    return excl;
}

// ------------------------------------------------------- predict + clamp
// KIntegratePred (sim/integrate.cu:40-51) followed by the position half of
// KBoundary with e = 0 (sim/boundary.cu:11-25): v' = v + g dt (fused),
// x = p + v' dt (fused), clamp min-then-max per axis, w = 1.  The explicit
// __fmaf_rn pins the rounding so cell keys are reproducible bit for bit.
__device__ __forceinline__ float4 predict_clamped(float4 p, float4 v, float3 g, float dt, const sim::GridBounds& gb) {
    float vx = __fmaf_rn(g.x, dt, v.x);
    float vy = __fmaf_rn(g.y, dt, v.y);
    float vz = __fmaf_rn(g.z, dt, v.z);
    float x = __fmaf_rn(vx, dt, p.x);
    float y = __fmaf_rn(vy, dt, p.y);
    float z = __fmaf_rn(vz, dt, p.z);
    if (x < gb.mins.x) x = gb.mins.x;
    if (y < gb.mins.y) y = gb.mins.y;
    if (z < gb.mins.z) z = gb.mins.z;
    if (x > gb.maxs.x) x = gb.maxs.x;
    if (y > gb.maxs.y) y = gb.maxs.y;
    if (z > gb.maxs.z) z = gb.maxs.z;
    return make_float4(x, y, z, 1.0f);
}

// Full KBoundary on a (position, velocity) pair (sim/boundary.cu:11-25).
__device__ __forceinline__ void boundary_apply(float4& p, float4& v, const sim::GridBounds& gb, float restitution) {
    const float e = fminf(fmaxf(restitution, 0.0f), 1.0f);
    if (p.x < gb.mins.x) { p.x = gb.mins.x; v.x *= -e; }
    if (p.y < gb.mins.y) { p.y = gb.mins.y; v.y *= -e; }
    if (p.z < gb.mins.z) { p.z = gb.mins.z; v.z *= -e; }
    if (p.x > gb.maxs.x) { p.x = gb.maxs.x; v.x *= -e; }
    if (p.y > gb.maxs.y) { p.y = gb.maxs.y; v.y *= -e; }
    if (p.z > gb.maxs.z) { p.z = gb.maxs.z; v.z *= -e; }
    p.w = 1.0f;
    v.w = 0.0f;
}

// KHash (sim/hash_keys.cu:6-27): IEEE divide, floor, clamp to [0,dim-1],
// key = (z*Y + y)*X + x.
__device__ __forceinline__ uint32_t cell_key(float4 p, const sim::GridBounds& gb) {
    int cx = __float2int_rz(floorf(__fdiv_rn(p.x - gb.mins.x, gb.cellSize)));
    int cy = __float2int_rz(floorf(__fdiv_rn(p.y - gb.mins.y, gb.cellSize)));
    int cz = __float2int_rz(floorf(__fdiv_rn(p.z - gb.mins.z, gb.cellSize)));
    cx = max(0, min(cx, gb.dim.x - 1));
    cy = max(0, min(cy, gb.dim.y - 1));
    cz = max(0, min(cz, gb.dim.z - 1));
    return uint32_t((cz * gb.dim.y + cy) * gb.dim.x + cx);
}

__device__ __forceinline__ void decode_key(uint32_t key, int3 dim, int& cx, int& cy, int& cz) {
    cx = int(key % uint32_t(dim.x));
    const uint32_t kdx = key / uint32_t(dim.x);
    cy = int(kdx % uint32_t(dim.y));
    cz = int(kdx / uint32_t(dim.y));
}

// reach = max(1, ceil(h / cs)) (sim/pbf_lambda.cu:47).
__device__ __forceinline__ int neighbour_reach(const sim::DeviceParams& dp) {
    const float cs = dp.grid.cellSize;
    return (cs > 0.f) ? max(1, int(ceilf(dp.kernel.h / cs))) : 1;
}

// Enumerates the (2*reach+1)^2 rows of the stencil in reference order and
// calls visit(k) for every candidate slot k.  rowRange(firstCell, lastCell)
// returns the contiguous slot range [b,e) covering those cells.
template <class RowRange, class Visit>
__device__ __forceinline__ void walk_neighbours(int cx, int cy, int cz, int reach, int3 dim, RowRange&& rowRange,
                                                Visit&& visit) {
    const int x0 = max(cx - reach, 0);
    const int x1 = min(cx + reach, dim.x - 1);
    for (int dz = -reach; dz <= reach; ++dz) {
        const int z = cz + dz;
        if (z < 0 || z >= dim.z) continue;
        for (int dy = -reach; dy <= reach; ++dy) {
            const int y = cy + dy;
            if (y < 0 || y >= dim.y) continue;
            const uint32_t row = uint32_t((z * dim.y + y) * dim.x);
            uint2 r = rowRange(row + uint32_t(x0), row + uint32_t(x1));
            for (uint32_t k = r.x; k < r.y; ++k)
                if (!visit(k)) return;
        }
    }
}

// Row ranges from a dense lower-bound table lb[c] = first sorted slot whose
// key >= c (numCells+1 entries).
struct LbRows {
    const uint32_t* __restrict__ lb;
    __device__ __forceinline__ uint2 operator()(uint32_t c0, uint32_t c1) const {
        return make_uint2(__ldg(lb + c0), __ldg(lb + c1 + 1u));
    }
};

// Row ranges from the reference's dense table (start = 0xFFFFFFFF and
// end = 0 for empty cells): min of starts, max of ends.
struct DenseRows {
    const uint32_t* __restrict__ start;
    const uint32_t* __restrict__ end;
    __device__ __forceinline__ uint2 operator()(uint32_t c0, uint32_t c1) const {
        uint32_t b = 0xFFFFFFFFu, e = 0u;
        for (uint32_t c = c0; c <= c1; ++c) {
            uint32_t s = __ldg(start + c), t = __ldg(end + c);
            if (s != 0xFFFFFFFFu && s < t) {
                b = min(b, s);
                e = max(e, t);
            }
        }
        if (b == 0xFFFFFFFFu) b = e = 0u;
        return make_uint2(b, e);
    }
};

// Row ranges from the reference's compact table (sorted unique keys,
// offsets): lower_bound of the first cell (sim/cuda_grid_utils.cuh:34-67),
// then forward over the segments inside the row.
struct CompactRows {
    const uint32_t* __restrict__ uk;
    const uint32_t* __restrict__ off;
    uint32_t M;
    __device__ __forceinline__ uint2 operator()(uint32_t c0, uint32_t c1) const {
        uint32_t lo = 0, hi = M;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (__ldg(uk + mid) < c0) lo = mid + 1; else hi = mid;
        }
        uint32_t m = lo;
        while (m < M && __ldg(uk + m) <= c1) ++m;
        if (m == lo) return make_uint2(0u, 0u);
        return make_uint2(__ldg(off + lo), __ldg(off + m));
    }
};

// ---------------------------------------------------------------- lambda
// Per-particle constraint multiplier, sim/pbf_lambda.cu:38-107.  fetch(k)
// returns the candidate's identity (compared with `self`) and position.
template <class RowRange, class Fetch>
__device__ __forceinline__ float lambda_of(uint32_t self, float4 pi, int cx, int cy, int cz,
                                           const sim::DeviceParams& dp, RowRange&& rows, Fetch&& fetch) {
    const sim::KernelCoeffs& kc = dp.kernel;
    const sim::PbfTuning& pbf = dp.pbf;
    const float particleMass = dp.particleMass;
    const float restDensity = dp.restDensity;
    float density = 0.f, gx = 0.f, gy = 0.f, gz = 0.f, sumGrad2 = 0.f;
    int contrib = 0;
    const int cap = dp.maxNeighbors;
    const bool hasCap = cap > 0;
    walk_neighbours(cx, cy, cz, neighbour_reach(dp), dp.grid.dim, rows, [&](uint32_t k) -> bool {
        if (hasCap && contrib >= cap) return false;
        uint32_t j;
        const float4 pj = fetch(k, j);
        if (j == self) return true;
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = rx * rx + ry * ry + rz * rz;
        if (r2 > kc.h2) return true;
        ++contrib;
        const float hr2 = kc.h2 - r2;
        density += particleMass * kc.poly6 * hr2 * hr2 * hr2;
        const float r = sqrtf(r2);
        const float r_safe = fmaxf(r, pbf.grad_r_eps);
        const float t = kc.h - r;
        const float coeff = (-3.0f * kc.spiky * (t * t) / r_safe);
        const float ax = coeff * rx, ay = coeff * ry, az = coeff * rz;
        gx += ax; gy += ay; gz += az;
        sumGrad2 += ax * ax + ay * ay + az * az;
        return true;
    });
    const float gradSum2 = gx * gx + gy * gy + gz * gz;
    const float scale = (restDensity > 0.f) ? (particleMass / restDensity) : 0.f;
    float denom = (scale * scale) * (sumGrad2 + gradSum2) + pbf.lambda_denom_eps;
    if (pbf.compliance > 0.f && dp.dt > 0.f) denom += pbf.compliance / (dp.dt * dp.dt);
    denom = fmaxf(denom, pbf.lambda_denom_eps);
    if (contrib < 2 || (sumGrad2 + gradSum2) < 1e-12f) return 0.0f;
    const float C = (restDensity > 0.f) ? (density / restDensity - 1.f) : 0.f;
    float lam = -C / denom;
    if (!isfinite(lam)) lam = 0.f;
    if (pbf.enable_lambda_clamp) {
        if (fabsf(lam) > pbf.lambda_max_abs) lam = copysignf(pbf.lambda_max_abs, lam);
    }
    return lam;
}

// s_corr exponent: powf, as the reference (sim/pbf_delta_apply.cu:82).
__device__ __forceinline__ float scorr_pow(float ratio, float n) { return powf(ratio, n); }

// w_q of the tensile-instability term (sim/pbf_delta_apply.cu:40-42).
__device__ __forceinline__ float scorr_wq(const sim::DeviceParams& dp) {
    const float dq = dp.pbf.scorr_dq_h * dp.kernel.h;
    const float hr2_q = dp.kernel.h2 - dq * dq;
    return (hr2_q > 0.f) ? (dp.kernel.poly6 * hr2_q * hr2_q * hr2_q) : dp.pbf.wq_min;
}

// ----------------------------------------------------------------- delta
// Position correction, sim/pbf_delta_apply.cu:40-112.  fetch(k, j, lam_j)
// returns the candidate position and writes its identity and lambda.
template <class RowRange, class Fetch>
__device__ __forceinline__ float3 delta_of(uint32_t self, float4 pi, float lam_i, int cx, int cy, int cz,
                                           const sim::DeviceParams& dp, float w_q, RowRange&& rows, Fetch&& fetch) {
    const sim::KernelCoeffs& kc = dp.kernel;
    const sim::PbfTuning& pbf = dp.pbf;
    float dx = 0.f, dy = 0.f, dz = 0.f;
    walk_neighbours(cx, cy, cz, neighbour_reach(dp), dp.grid.dim, rows, [&](uint32_t k) -> bool {
        uint32_t j;
        float lam_j;
        const float4 pj = fetch(k, j, lam_j);
        if (j == self) return true;
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = rx * rx + ry * ry + rz * rz;
        if (r2 > kc.h2) return true;
        const float r = sqrtf(r2);
        const float t = kc.h - r;
        const float r_safe = fmaxf(r, pbf.grad_r_eps);
        const float coeff = (-3.0f * kc.spiky * (t * t) / r_safe);
        const float ax = coeff * rx, ay = coeff * ry, az = coeff * rz;
        float scorr = 0.0f;
        if (pbf.scorr_enable) {
            const float hr2 = kc.h2 - r2;
            const float w = kc.poly6 * hr2 * hr2 * hr2;
            const float ratio = (w_q > 0.f) ? (w / w_q) : 0.0f;
            scorr = -pbf.scorr_k * scorr_pow(ratio, pbf.scorr_n);
            if (pbf.scorr_min < 0.f) scorr = fmaxf(scorr, pbf.scorr_min);
        }
        const float lij = (lam_i + lam_j + scorr);
        dx += lij * ax;
        dy += lij * ay;
        dz += lij * az;
        return true;
    });
    const float invRest = (dp.restDensity > 0.f) ? (1.0f / dp.restDensity) : 0.f;
    float3 d = make_float3(invRest * dx, invRest * dy, invRest * dz);
    if (pbf.enable_relax) {
        d.x *= pbf.relax_omega;
        d.y *= pbf.relax_omega;
        d.z *= pbf.relax_omega;
    }
    if (pbf.enable_disp_clamp) {
        const float maxDisp = pbf.disp_clamp_max_h * kc.h;
        const float maxDisp2 = maxDisp * maxDisp;
        const float len2 = d.x * d.x + d.y * d.y + d.z * d.z;
        if (len2 > maxDisp2) {
            const float len = sqrtf(len2);
            const float s = maxDisp / (len + 1e-20f);
            d.x *= s; d.y *= s; d.z *= s;
        }
    }
    return d;
}

// ------------------------------------------------------------------ xsph
// Jacobi XSPH, sim/xsph.cu:39-95.  fetch(k, j, vj) returns the candidate
// position and writes its identity and (old) velocity.
template <class RowRange, class Fetch>
__device__ __forceinline__ float4 xsph_of(uint32_t self, float4 pi, float4 vi, int cx, int cy, int cz,
                                          const sim::DeviceParams& dp, RowRange&& rows, Fetch&& fetch) {
    const sim::KernelCoeffs& kc = dp.kernel;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    int count = 0;
    walk_neighbours(cx, cy, cz, neighbour_reach(dp), dp.grid.dim, rows, [&](uint32_t k) -> bool {
        uint32_t j;
        float4 vj;
        const float4 pj = fetch(k, j, vj);
        if (j == self) return true;
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = rx * rx + ry * ry + rz * rz;
        if (r2 > kc.h2) return true;
        const float hr2 = kc.h2 - r2;
        const float w = kc.poly6 * hr2 * hr2 * hr2;
        sx += (vj.x - vi.x) * w;
        sy += (vj.y - vi.y) * w;
        sz += (vj.z - vi.z) * w;
        ++count;
        return true;
    });
    float gate = 1.0f;
    if (dp.pbf.xsph_gate_enable) {
        const int nMin = max(0, dp.pbf.xsph_n_min);
        const int nMax = max(nMin + 1, dp.pbf.xsph_n_max);
        const float t = (float(count) - float(nMin)) / float(nMax - nMin);
        gate = fminf(1.f, fmaxf(0.f, t));
    }
    const float mor = (dp.restDensity > 0.f) ? (dp.particleMass / dp.restDensity) : 0.f;
    return make_float4(vi.x + (dp.xsph_c * gate) * mor * sx, vi.y + (dp.xsph_c * gate) * mor * sy,
                       vi.z + (dp.xsph_c * gate) * mor * sz, 0.0f);
}

// Grid size helper.
inline unsigned blocks_for(uint64_t n, unsigned bs) { return unsigned((n + bs - 1) / bs); }

}  // namespace pbf
