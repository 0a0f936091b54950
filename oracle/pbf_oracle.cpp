// pbf_oracle.cpp - CPU restatement of the reference PBF step (test checker).
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py; never by the product library.
//
// Build: g++ -O3 -std=c++17 -fopenmp -ffp-contract=off -shared -fPIC
// (no fast-math, no implicit contraction: results are identical on x86-64
// and aarch64).  Templated on the real type: float reproduces the
// reference's FP32 arithmetic op for op, double is the FP64 oracle.
//
// FMA contraction.  nvcc (default -fmad=true) fuses some multiply-adds of the
// reference kernels; the fused operations are written out here as explicit
// fma calls, so the FP32 oracle reproduces the reference kernels bit for bit.
// The fused sites were identified by comparing candidate forms against the
// reference kernels' outputs on the GPU (32,768 particles, lattice and
// compressed states; every lambda and XSPH velocity bit-identical):
//   r^2 = fma(rz, rz, fma(rx, rx, ry*ry))               all neighbour loops
//   density = fma(m*poly6*hr2*hr2, hr2, density)         lambda
//   sumGrad2 = sumGrad2 + fma(az, az, fma(ax, ax, ay*ay)) lambda (gradSum += a unfused)
//   |gradSum|^2 like r^2; denom = fma(scale*scale, sum, eps)
//   dx = fma(lij, ax, dx); |d|^2 like r^2;  w_q: h2 - dq*dq = fma(-dq, dq, h2)   delta
//   sum = fma(vj - vi, W, sum); v = fma(c*gate*m/rho0, sum, vi)                  XSPH
// The one operation the oracle cannot reproduce exactly is CUDA's powf (the
// s_corr exponent), which is not correctly rounded; the oracle uses the C
// library's powf, so position corrections agree to rounding, not bitwise.
#include "pbf_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename R>
struct V3 {
    R x, y, z;
};

template <typename R>
struct V4 {
    R x, y, z, w;
};

// Real-typed copy of pbf_device_params (float: the same values).
template <typename R>
struct P {
    R h, h2, poly6, spiky;
    V3<R> mins, maxs;
    R cs;
    int dimx, dimy, dimz;
    V3<R> g;
    R rest, dt, inv_dt, e, mass, xsph_c;
    int maxNeighbors;
    // tuning
    int scorr_enable;
    R scorr_k, scorr_n, scorr_dq_h, wq_min, scorr_min, grad_r_eps, lambda_denom_eps, compliance;
    int enable_lambda_clamp;
    R lambda_max_abs;
    int enable_disp_clamp;
    R disp_clamp_max_h;
    int enable_relax;
    R relax_omega;
    int xsph_gate_enable, xsph_n_min, xsph_n_max;
};

template <typename R>
P<R> make_p(const pbf_device_params& d) {
    P<R> p{};
    p.h = R(d.kernel.h);
    p.h2 = R(d.kernel.h2);
    p.poly6 = R(d.kernel.poly6);
    p.spiky = R(d.kernel.spiky);
    p.mins = {R(d.grid.mins.x), R(d.grid.mins.y), R(d.grid.mins.z)};
    p.maxs = {R(d.grid.maxs.x), R(d.grid.maxs.y), R(d.grid.maxs.z)};
    p.cs = R(d.grid.cellSize);
    p.dimx = d.grid.dim.x;
    p.dimy = d.grid.dim.y;
    p.dimz = d.grid.dim.z;
    p.g = {R(d.gravity.x), R(d.gravity.y), R(d.gravity.z)};
    p.rest = R(d.restDensity);
    p.dt = R(d.dt);
    p.inv_dt = R(d.inv_dt);
    p.e = R(d.boundaryRestitution);
    p.mass = R(d.particleMass);
    p.xsph_c = R(d.xsph_c);
    p.maxNeighbors = d.maxNeighbors;
    const pbf_tuning& t = d.pbf;
    p.scorr_enable = t.scorr_enable;
    p.scorr_k = R(t.scorr_k);
    p.scorr_n = R(t.scorr_n);
    p.scorr_dq_h = R(t.scorr_dq_h);
    p.wq_min = R(t.wq_min);
    p.scorr_min = R(t.scorr_min);
    p.grad_r_eps = R(t.grad_r_eps);
    p.lambda_denom_eps = R(t.lambda_denom_eps);
    p.compliance = R(t.compliance);
    p.enable_lambda_clamp = t.enable_lambda_clamp;
    p.lambda_max_abs = R(t.lambda_max_abs);
    p.enable_disp_clamp = t.enable_disp_clamp;
    p.disp_clamp_max_h = R(t.disp_clamp_max_h);
    p.enable_relax = t.enable_relax;
    p.relax_omega = R(t.relax_omega);
    p.xsph_gate_enable = t.xsph_gate_enable;
    p.xsph_n_min = t.xsph_n_min;
    p.xsph_n_max = t.xsph_n_max;
    return p;
}

// FP64 oracle kernel constants are recomputed in double from the same h so
// that poly6/spiky carry no FP32 rounding.
P<double> make_p64(const pbf_device_params& d) {
    P<double> p = make_p<double>(d);
    const double pi = 3.14159265358979323846;
    const double h = p.h;
    p.h2 = h * h;
    p.poly6 = 315.0 / (64.0 * pi * std::pow(h, 9));
    p.spiky = 15.0 / (pi * std::pow(h, 6));
    p.inv_dt = (p.dt > 0) ? 1.0 / p.dt : 0.0;
    return p;
}

inline float4 f4(float x, float y, float z, float w) {
    float4 r;
    r.x = x; r.y = y; r.z = z; r.w = w;
    return r;
}

inline float fma_r(float a, float b, float c) { return std::fmaf(a, b, c); }
inline double fma_r(double a, double b, double c) { return std::fma(a, b, c); }

// The real-type operations of the kernels below, overloaded per type (float,
// double, and the dual numbers of the forward-mode derivative further down).
// max_r is std::max's (a < b) ? b : a.
inline float floor_r(float a) { return std::floor(a); }
inline double floor_r(double a) { return std::floor(a); }
inline float sqrt_r(float a) { return std::sqrt(a); }
inline double sqrt_r(double a) { return std::sqrt(a); }
template <typename R>
inline R max_r(R a, R b) { return (a < b) ? b : a; }
inline bool isfinite_r(float a) { return std::isfinite(a); }
inline bool isfinite_r(double a) { return std::isfinite(a); }
inline float fabs_r(float a) { return std::fabs(a); }
inline double fabs_r(double a) { return std::fabs(a); }
inline float copysign_r(float a, float b) { return std::copysign(a, b); }
inline double copysign_r(double a, double b) { return std::copysign(a, b); }

// sim/integrate.cu:40-51 (KIntegratePred).  The GPU computes both
// multiply-adds as single fused operations; fmaf reproduces them exactly.
template <typename R>
void integrate_pred_t(const V4<R>* pos, const V4<R>* vel, V4<R>* pred, V3<R> g, R dt, uint32_t N) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        V4<R> p = pos[i], v = vel[i];
        R vx = fma_r(g.x, dt, v.x);
        R vy = fma_r(g.y, dt, v.y);
        R vz = fma_r(g.z, dt, v.z);
        pred[i] = {fma_r(vx, dt, p.x), fma_r(vy, dt, p.y), fma_r(vz, dt, p.z), p.w};
    }
}

// sim/boundary.cu:11-25 (KBoundary): min checks x,y,z then max checks x,y,z.
template <typename R>
void boundary_t(V4<R>* pred, V4<R>* vel, V3<R> mins, V3<R> maxs, R restitution, uint32_t N) {
    R e = restitution;
    if (e < R(0)) e = R(0);
    if (e > R(1)) e = R(1);
    // fminf(fmaxf(r,0),1) also maps NaN to 0
    if (!(restitution == restitution)) e = R(0);
    const R ne = -e;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        V4<R> p = pred[i], v = vel[i];
        if (p.x < mins.x) { p.x = mins.x; v.x *= ne; }
        if (p.y < mins.y) { p.y = mins.y; v.y *= ne; }
        if (p.z < mins.z) { p.z = mins.z; v.z *= ne; }
        if (p.x > maxs.x) { p.x = maxs.x; v.x *= ne; }
        if (p.y > maxs.y) { p.y = maxs.y; v.y *= ne; }
        if (p.z > maxs.z) { p.z = maxs.z; v.z *= ne; }
        pred[i] = {p.x, p.y, p.z, R(1)};
        vel[i] = {v.x, v.y, v.z, R(0)};
    }
}

// sim/boundary.cu:28-34 (KVelocity).
template <typename R>
void velocity_t(V4<R>* vel, const V4<R>* pos, const V4<R>* pred, R inv_dt, uint32_t N) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        vel[i] = {(pred[i].x - pos[i].x) * inv_dt, (pred[i].y - pos[i].y) * inv_dt,
                  (pred[i].z - pos[i].z) * inv_dt, R(0)};
    }
}

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// float -> int as the GPU's truncating conversion: NaN -> 0, saturating.
template <typename R>
inline int to_int_sat(R f) {
    if (!(f == f)) return 0;
    if (f >= R(2147483647.0)) return 2147483647;
    if (f <= R(-2147483648.0)) return (-2147483647 - 1);
    return (int)f;
}

// sim/hash_keys.cu:6-27 (linearIndex + KHash): IEEE divide, floor, clamp.
template <typename R>
void hash_keys_t(uint32_t* keys, uint32_t* idx, const V4<R>* pred, V3<R> mins, R cs, int dx, int dy,
                 int dz, uint32_t N) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        R rx = (pred[i].x - mins.x) / cs;
        R ry = (pred[i].y - mins.y) / cs;
        R rz = (pred[i].z - mins.z) / cs;
        int cx = clampi(to_int_sat(floor_r(rx)), 0, dx - 1);
        int cy = clampi(to_int_sat(floor_r(ry)), 0, dy - 1);
        int cz = clampi(to_int_sat(floor_r(rz)), 0, dz - 1);
        keys[i] = (uint32_t)((cz * dy + cy) * dx + cx);
        if (idx) idx[i] = (uint32_t)i;
    }
}

// Reference cell lookups.  Dense: sim/phases.cpp + sim/cell_ranges.cu
// semantics (start==0xFFFFFFFF or start>=end means empty).  Compact:
// lower_bound on unique keys (sim/cuda_grid_utils.cuh:34-67).
struct Table {
    const uint32_t* start;
    const uint32_t* end;
    const uint32_t* uk;
    const uint32_t* off;
    uint32_t M;
    bool lookup(uint32_t cidx, uint32_t& b, uint32_t& e) const {
        if (!uk) {
            b = start[cidx];
            e = end[cidx];
            return !(b == 0xFFFFFFFFu || b >= e);
        }
        if (M == 0) { b = e = 0; return false; }
        uint32_t lo = 0, hi = M;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (uk[mid] < cidx) lo = mid + 1; else hi = mid;
        }
        if (lo >= M || uk[lo] != cidx) { b = e = 0; return false; }
        b = off[lo];
        e = off[lo + 1];
        return b < e;
    }
};

Table make_table(const oracle_table* t) {
    Table tb{};
    tb.start = t->start;
    tb.end = t->end;
    tb.uk = t->unique_keys;
    tb.off = t->offsets;
    tb.M = t->count;
    return tb;
}

template <typename R>
inline void decode(uint32_t key, const P<R>& p, int& cx, int& cy, int& cz) {
    cx = int(key % uint32_t(p.dimx));
    uint32_t kdx = key / uint32_t(p.dimx);
    cy = int(kdx % uint32_t(p.dimy));
    cz = int(kdx / uint32_t(p.dimy));
}

template <typename R>
inline int reach_of(const P<R>& p) {
    if (!(p.cs > R(0))) return 1;
    int r = int(std::ceil(float(p.h) / float(p.cs)));  // ceilf(h / cs) in FP32
    return r > 1 ? r : 1;
}

// Neighbour iteration in reference order (sim/pbf_lambda.cu:49-84): for a
// particle in cell (cx,cy,cz): dz, dy, dx in [-reach, reach], cells outside
// [0,dim) skipped, then k ascending over the cell's sorted range.  f returns
// false to stop the whole walk.
template <typename R, typename F>
inline void for_candidates(int cx, int cy, int cz, int reach, const P<R>& p, const Table& tb, F&& f) {
    for (int dz = -reach; dz <= reach; ++dz)
        for (int dy = -reach; dy <= reach; ++dy)
            for (int dx = -reach; dx <= reach; ++dx) {
                int x = cx + dx, y = cy + dy, z = cz + dz;
                if (x < 0 || y < 0 || z < 0 || x >= p.dimx || y >= p.dimy || z >= p.dimz) continue;
                uint32_t cidx = (uint32_t)((z * p.dimy + y) * p.dimx + x);
                uint32_t b, e;
                if (!tb.lookup(cidx, b, e)) continue;
                for (uint32_t k = b; k < e; ++k)
                    if (!f(k)) return;
            }
}

// sim/pbf_lambda.cu:10-108 (KLambdaGlobalsDense / Compact).
template <typename R>
void lambda_t(R* lambda, const V4<R>* pred, const uint32_t* idx, const uint32_t* keys, const Table& tb,
              const P<R>& p, uint32_t N) {
    const int reach = reach_of(p);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t s = 0; s < (int64_t)N; ++s) {
        const uint32_t i = idx[s];
        const V4<R> pi = pred[i];
        int cx, cy, cz;
        decode(keys[s], p, cx, cy, cz);
        R density = 0, gx = 0, gy = 0, gz = 0, sumGrad2 = 0;
        int contrib = 0;
        const int cap = p.maxNeighbors;
        const bool hasCap = cap > 0;
        for_candidates(cx, cy, cz, reach, p, tb, [&](uint32_t k) -> bool {
            if (hasCap && contrib >= cap) return false;
            const uint32_t j = idx[k];
            if (j == i) return true;
            const V4<R> pj = pred[j];
            R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            R r2 = fma_r(rz, rz, fma_r(rx, rx, ry * ry));
            if (r2 > p.h2) return true;
            ++contrib;
            R hr2 = p.h2 - r2;
            density = fma_r(p.mass * p.poly6 * hr2 * hr2, hr2, density);
            R r = sqrt_r(r2);
            R r_safe = max_r(r, p.grad_r_eps);
            R t = p.h - r;
            R coeff = (R(-3) * p.spiky * (t * t) / r_safe);
            R ax = coeff * rx, ay = coeff * ry, az = coeff * rz;
            gx += ax; gy += ay; gz += az;
            sumGrad2 = sumGrad2 + fma_r(az, az, fma_r(ax, ax, ay * ay));
            return true;
        });
        R gradSum2 = fma_r(gz, gz, fma_r(gx, gx, gy * gy));
        R scale = (p.rest > R(0)) ? (p.mass / p.rest) : R(0);
        R denom = fma_r(scale * scale, sumGrad2 + gradSum2, p.lambda_denom_eps);
        if (p.compliance > R(0) && p.dt > R(0)) denom += p.compliance / (p.dt * p.dt);
        denom = max_r(denom, p.lambda_denom_eps);
        R lam;
        if (contrib < 2 || (sumGrad2 + gradSum2) < R(1e-12f)) {
            lam = R(0);
        } else {
            R C = (p.rest > R(0)) ? (density / p.rest - R(1)) : R(0);
            lam = -C / denom;
            if (!isfinite_r(lam)) lam = R(0);
            if (p.enable_lambda_clamp) {
                if (fabs_r(lam) > p.lambda_max_abs) lam = copysign_r(p.lambda_max_abs, lam);
            }
        }
        lambda[i] = lam;
    }
}

inline float pow_r(float a, float b) { return std::pow(a, b); }
inline double pow_r(double a, double b) { return std::pow(a, b); }

// sim/pbf_delta_apply.cu:10-113 (KDeltaCompute) + :223-235 (KApplyDelta).
template <typename R>
void delta_apply_t(V4<R>* pred, V4<R>* delta, const R* lambda, const uint32_t* idx, const uint32_t* keys,
                   const Table& tb, const P<R>& p, uint32_t N) {
    const int reach = reach_of(p);
    const R dq = p.scorr_dq_h * p.h;
    const R hr2_q = fma_r(-dq, dq, p.h2);
    const R w_q = (hr2_q > R(0)) ? (p.poly6 * hr2_q * hr2_q * hr2_q) : p.wq_min;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t s = 0; s < (int64_t)N; ++s) {
        const uint32_t i = idx[s];
        const V4<R> pi = pred[i];
        int cx, cy, cz;
        decode(keys[s], p, cx, cy, cz);
        R dx_ = 0, dy_ = 0, dz_ = 0;
        for_candidates(cx, cy, cz, reach, p, tb, [&](uint32_t k) -> bool {
            const uint32_t j = idx[k];
            if (j == i) return true;
            const V4<R> pj = pred[j];
            R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            R r2 = fma_r(rz, rz, fma_r(rx, rx, ry * ry));
            if (r2 > p.h2) return true;
            R r = sqrt_r(r2);
            R t = p.h - r;
            R r_safe = max_r(r, p.grad_r_eps);
            R coeff = (R(-3) * p.spiky * (t * t) / r_safe);
            R ax = coeff * rx, ay = coeff * ry, az = coeff * rz;
            R scorr = 0;
            if (p.scorr_enable) {
                R hr2 = p.h2 - r2;
                R w = p.poly6 * hr2 * hr2 * hr2;
                R ratio = (w_q > R(0)) ? (w / w_q) : R(0);
                scorr = -p.scorr_k * pow_r(ratio, p.scorr_n);
                if (p.scorr_min < R(0)) scorr = max_r(scorr, p.scorr_min);
            }
            R lij = (lambda[i] + lambda[j] + scorr);
            dx_ = fma_r(lij, ax, dx_);
            dy_ = fma_r(lij, ay, dy_);
            dz_ = fma_r(lij, az, dz_);
            return true;
        });
        R invRest = (p.rest > R(0)) ? (R(1) / p.rest) : R(0);
        R ex = invRest * dx_, ey = invRest * dy_, ez = invRest * dz_;
        if (p.enable_relax) { ex *= p.relax_omega; ey *= p.relax_omega; ez *= p.relax_omega; }
        if (p.enable_disp_clamp) {
            R maxDisp = p.disp_clamp_max_h * p.h;
            R maxDisp2 = maxDisp * maxDisp;
            R len2 = fma_r(ez, ez, fma_r(ex, ex, ey * ey));
            if (len2 > maxDisp2) {
                R len = sqrt_r(len2);
                R sc = maxDisp / (len + R(1e-20f));
                ex *= sc; ey *= sc; ez *= sc;
            }
        }
        delta[i] = {ex, ey, ez, R(0)};
    }
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < (int64_t)N; ++s) {
        const uint32_t i = idx[s];
        V4<R> b = pred[i];
        pred[i] = {b.x + delta[i].x, b.y + delta[i].y, b.z + delta[i].z, b.w};
    }
}

// sim/xsph.cu:9-96 (KXSPH), Jacobi: reads vel_in only.
template <typename R>
void xsph_t(V4<R>* vel_out, const V4<R>* vel_in, const V4<R>* pred, const uint32_t* idx, const uint32_t* keys,
            const Table& tb, const P<R>& p, uint32_t N) {
    const int reach = reach_of(p);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t s = 0; s < (int64_t)N; ++s) {
        const uint32_t i = idx[s];
        const V4<R> pi = pred[i];
        const V4<R> vi = vel_in[i];
        int cx, cy, cz;
        decode(keys[s], p, cx, cy, cz);
        R sx = 0, sy = 0, sz = 0;
        int count = 0;
        for_candidates(cx, cy, cz, reach, p, tb, [&](uint32_t k) -> bool {
            const uint32_t j = idx[k];
            if (j == i) return true;
            const V4<R> pj = pred[j];
            R rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            R r2 = fma_r(rz, rz, fma_r(rx, rx, ry * ry));
            if (r2 > p.h2) return true;
            R hr2 = p.h2 - r2;
            R w = p.poly6 * hr2 * hr2 * hr2;
            const V4<R> vj = vel_in[j];
            sx = fma_r(vj.x - vi.x, w, sx);
            sy = fma_r(vj.y - vi.y, w, sy);
            sz = fma_r(vj.z - vi.z, w, sz);
            ++count;
            return true;
        });
        R gate = 1;
        if (p.xsph_gate_enable) {
            int nMin = std::max(0, p.xsph_n_min);
            int nMax = std::max(nMin + 1, p.xsph_n_max);
            float t = (float(count) - float(nMin)) / float(nMax - nMin);
            gate = R(std::min(1.f, std::max(0.f, t)));
        }
        R mor = (p.rest > R(0)) ? (p.mass / p.rest) : R(0);
        R c = (p.xsph_c * gate) * mor;
        vel_out[i] = {fma_r(c, sx, vi.x), fma_r(c, sy, vi.y), fma_r(c, sz, vi.z), R(0)};
    }
}

// Stable LSD radix sort of (key, value) over bits [0,32): the same order as
// the reference's cub::DeviceRadixSort::SortPairs (sim/sort_pairs.cu:18-27).
void sort_pairs_impl(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t N) {
    std::vector<uint32_t> k0(kin, kin + N), v0(vin, vin + N), k1(N), v1(N);
    for (int pass = 0; pass < 4; ++pass) {
        const int sh = pass * 8;
        size_t cnt[257] = {0};
        for (uint32_t i = 0; i < N; ++i) cnt[((k0[i] >> sh) & 255u) + 1]++;
        bool trivial = false;
        for (int d = 0; d < 256; ++d)
            if (cnt[d + 1] == N) trivial = true;
        if (trivial) continue;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (uint32_t i = 0; i < N; ++i) {
            size_t pos = cnt[(k0[i] >> sh) & 255u]++;
            k1[pos] = k0[i];
            v1[pos] = v0[i];
        }
        k0.swap(k1);
        v0.swap(v1);
    }
    std::memcpy(kout, k0.data(), sizeof(uint32_t) * N);
    std::memcpy(vout, v0.data(), sizeof(uint32_t) * N);
}

// sim/cell_ranges.cu:21-51 with the memsets of sim/phases.cpp:58-59 and
// sim/cell_ranges.cu:62-63 (start=0xFFFFFFFF, end=0 for empty cells).
void cell_ranges_impl(uint32_t* start, uint32_t* end, const uint32_t* ks, uint32_t N, uint32_t numCells) {
    for (uint32_t c = 0; c < numCells; ++c) { start[c] = 0xFFFFFFFFu; end[c] = 0u; }
    for (uint32_t i = 0; i < N; ++i) {
        uint32_t k = ks[i];
        if (k >= numCells) continue;
        if (i == 0) start[k] = 0;
        else {
            uint32_t kp = ks[i - 1];
            if (k != kp) {
                if (kp < numCells) end[kp] = i;
                start[k] = i;
            }
        }
        if (i == N - 1) end[k] = N;
    }
}

// sim/cell_compact.cu:96-184 (flags, block scan, scatter + terminator).
void cell_compact_impl(uint32_t* uk, uint32_t* off, uint32_t* count, const uint32_t* ks, uint32_t N) {
    if (N == 0) { off[0] = 0; *count = 0; return; }
    uint32_t m = 0;
    for (uint32_t i = 0; i < N; ++i) {
        if (i == 0 || ks[i] != ks[i - 1]) {
            uk[m] = ks[i];
            off[m] = i;
            ++m;
        }
    }
    off[m] = N;
    *count = m;
}

inline const V4<float>* as4(const float4* p) { return reinterpret_cast<const V4<float>*>(p); }
inline V4<float>* as4(float4* p) { return reinterpret_cast<V4<float>*>(p); }

pbf_device_params device_params_of(const pbf_sim_params& sp) {
    pbf_device_params dp{};
    dp.kernel = sp.kernel;
    dp.grid = sp.grid;
    dp.gravity = sp.gravity;
    dp.restDensity = sp.restDensity;
    dp.dt = sp.dt;
    dp.inv_dt = (sp.dt > 0.f) ? (1.0f / sp.dt) : 0.0f;
    dp.boundaryRestitution = sp.boundaryRestitution;
    dp.maxNeighbors = sp.maxNeighbors;
    dp.particleMass = sp.particleMass;
    dp.pbf = sp.pbf;
    dp.xsph_c = sp.xsph_c;
    return dp;
}

// GridSystem::ComputeDims (sim/grid_system.h:9-17).
void compute_dims(pbf_grid_bounds& g) {
    const float cs = (g.cellSize > 0.f) ? g.cellSize : 1.f;
    int dx = int(std::ceil((g.maxs.x - g.mins.x) / cs));
    int dy = int(std::ceil((g.maxs.y - g.mins.y) / cs));
    int dz = int(std::ceil((g.maxs.z - g.mins.z) / cs));
    g.dim.x = dx < 0 ? 0 : dx;
    g.dim.y = dy < 0 ? 0 : dy;
    g.dim.z = dz < 0 ? 0 : dz;
}

// One step in reference order, generic over the real type.
template <typename R>
int step_t(const pbf_sim_params& sp0, int hashed, V4<R>* pos, V4<R>* vel, uint32_t N, oracle_trace* tr,
           const P<R>& p) {
    pbf_sim_params sp = sp0;
    compute_dims(sp.grid);
    const uint32_t numCells = uint32_t(sp.grid.dim.x) * uint32_t(sp.grid.dim.y) * uint32_t(sp.grid.dim.z);
    if (numCells == 0) return 1;
    std::vector<V4<R>> pred(N), delta(N), vtmp(N);
    std::vector<R> lam(N);
    std::vector<uint32_t> keys(N), idx(N), ks(N), is(N);
    // PhaseIntegrate (sim/phases.cpp:33-36)
    integrate_pred_t<R>(pos, vel, pred.data(), p.g, p.dt, N);
    boundary_t<R>(pred.data(), vel, p.mins, p.maxs, R(0), N);
    // PhaseGridBuildFull (sim/phases.cpp:44-63)
    hash_keys_t<R>(keys.data(), idx.data(), pred.data(), p.mins, p.cs, p.dimx, p.dimy, p.dimz, N);
    sort_pairs_impl(keys.data(), ks.data(), idx.data(), is.data(), N);
    std::vector<uint32_t> start, end, uk, off;
    uint32_t M = 0;
    Table tb{};
    if (hashed) {
        uk.resize(N > 0 ? N : 1);
        off.resize(N + 1);
        cell_compact_impl(uk.data(), off.data(), &M, ks.data(), N);
        tb.uk = uk.data();
        tb.off = off.data();
        tb.M = M;
    } else {
        start.resize(numCells);
        end.resize(numCells);
        cell_ranges_impl(start.data(), end.data(), ks.data(), N, numCells);
        tb.start = start.data();
        tb.end = end.data();
    }
    // PhaseSolveIterations (sim/phases.cpp:71-94)
    for (int it = 0; it < sp.solverIters; ++it) {
        lambda_t<R>(lam.data(), pred.data(), is.data(), ks.data(), tb, p, N);
        delta_apply_t<R>(pred.data(), delta.data(), lam.data(), is.data(), ks.data(), tb, p, N);
    }
    if (tr && tr->pred_solved) {
        for (uint32_t i = 0; i < N; ++i)
            tr->pred_solved[i] = f4(float(pred[i].x), float(pred[i].y), float(pred[i].z), float(pred[i].w));
    }
    boundary_t<R>(pred.data(), vel, p.mins, p.maxs, R(0), N);
    // PhaseVelocity (sim/phases.cpp:102-105): inv_dt = 1.0f / p.dt
    const R inv_dt = (sizeof(R) == 4) ? R(1.0f / sp.dt) : R(1.0) / R(p.dt);
    velocity_t<R>(vel, pos, pred.data(), inv_dt, N);
    if (tr && tr->vel_pre_xsph) {
        for (uint32_t i = 0; i < N; ++i)
            tr->vel_pre_xsph[i] = f4(float(vel[i].x), float(vel[i].y), float(vel[i].z), float(vel[i].w));
    }
    // PostOps XSPH -> Boundary -> Recycle (sim/post_ops.cpp:73-85)
    if (sp.xsph_c > 0.f) {
        xsph_t<R>(vtmp.data(), vel, pred.data(), is.data(), ks.data(), tb, p, N);
        std::memcpy(vel, vtmp.data(), sizeof(V4<R>) * N);
    }
    boundary_t<R>(pred.data(), vel, p.mins, p.maxs, p.e, N);
    // commit (ping-pong swap, sim/simulator.cpp:144-159)
    std::memcpy(pos, pred.data(), sizeof(V4<R>) * N);
    if (tr) {
        if (tr->keys) std::memcpy(tr->keys, keys.data(), 4 * N);
        if (tr->keys_sorted) std::memcpy(tr->keys_sorted, ks.data(), 4 * N);
        if (tr->perm) std::memcpy(tr->perm, is.data(), 4 * N);
        if (!hashed) {
            if (tr->cell_start) std::memcpy(tr->cell_start, start.data(), 4 * size_t(numCells));
            if (tr->cell_end) std::memcpy(tr->cell_end, end.data(), 4 * size_t(numCells));
        } else {
            if (tr->unique_keys) std::memcpy(tr->unique_keys, uk.data(), 4 * size_t(M));
            if (tr->offsets) std::memcpy(tr->offsets, off.data(), 4 * size_t(M + 1));
            if (tr->compact_count) *tr->compact_count = M;
        }
        if (tr->lambda)
            for (uint32_t i = 0; i < N; ++i) tr->lambda[i] = float(lam[i]);
    }
    return 0;
}

// FP64 density statistics over positions given as doubles.
void density_stats_impl(const pbf_sim_params& sp0, const double* xyz4, uint32_t N, double out[4]) {
    pbf_sim_params sp = sp0;
    compute_dims(sp.grid);
    pbf_device_params dp = device_params_of(sp);
    P<double> p = make_p64(dp);
    const uint32_t numCells = uint32_t(sp.grid.dim.x) * uint32_t(sp.grid.dim.y) * uint32_t(sp.grid.dim.z);
    std::vector<V4<double>> pos(N);
    for (uint32_t i = 0; i < N; ++i) pos[i] = {xyz4[4 * i], xyz4[4 * i + 1], xyz4[4 * i + 2], 1.0};
    std::vector<uint32_t> keys(N), idx(N), ks(N), is(N), start(numCells), end(numCells);
    // Cells from the FP32 positions' own rounding rules, evaluated in double.
    hash_keys_t<double>(keys.data(), idx.data(), pos.data(), p.mins, p.cs, p.dimx, p.dimy, p.dimz, N);
    sort_pairs_impl(keys.data(), ks.data(), idx.data(), is.data(), N);
    cell_ranges_impl(start.data(), end.data(), ks.data(), N, numCells);
    Table tb{};
    tb.start = start.data();
    tb.end = end.data();
    const int reach = reach_of(p);
    double sumAbs = 0, maxAbs = 0, sumPos = 0, sumNb = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : sumAbs, sumPos, sumNb) reduction(max : maxAbs)
    for (int64_t s = 0; s < (int64_t)N; ++s) {
        const uint32_t i = is[s];
        const V4<double> pi = pos[i];
        int cx, cy, cz;
        decode(ks[s], p, cx, cy, cz);
        double rho = 0;
        int nb = 0;
        for_candidates(cx, cy, cz, reach, p, tb, [&](uint32_t k) -> bool {
            const uint32_t j = is[k];
            if (j == i) return true;
            double rx = pi.x - pos[j].x, ry = pi.y - pos[j].y, rz = pi.z - pos[j].z;
            double r2 = rx * rx + ry * ry + rz * rz;
            if (r2 > p.h2) return true;
            double hr2 = p.h2 - r2;
            rho += p.mass * p.poly6 * hr2 * hr2 * hr2;
            ++nb;
            return true;
        });
        double C = (p.rest > 0) ? rho / p.rest - 1.0 : 0.0;
        sumAbs += std::fabs(C);
        maxAbs = std::max(maxAbs, std::fabs(C));
        sumPos += C > 0 ? C : 0.0;
        sumNb += nb;
    }
    const double n = N > 0 ? double(N) : 1.0;
    out[0] = sumAbs / n;
    out[1] = maxAbs;
    out[2] = sumPos / n;
    out[3] = sumNb / n;
}

// ----------------------------------------------- forward-mode derivative
// Dual numbers v + d e (e^2 = 0): running the step on them carries the exact
// directional derivative beside the value, with every branch (neighbour
// sets, caps, clamps, boundary) decided by the values, as the step itself
// decides it.  The derivative part is always FP64.  The value part is either
// FP64 (the derivative of the FP64 step) or FP32 (V = float: the values are
// the FP32 oracle's, i.e. the trajectory the GPU computes, up to the s_corr
// powf ulps, and the derivative is the FP64-accurate derivative along it,
// the reference tape of the adjoint's vector-Jacobian products).
template <class V>
struct DualT {
    V v;
    double d;
    DualT() = default;
    DualT(double x) : v(V(x)), d(0.0) {}  // NOLINT: constants and parameters
    DualT(V x, double dx, int) : v(x), d(dx) {}
    explicit operator float() const { return float(v); }
    explicit operator int() const { return int(v); }
    DualT& operator+=(const DualT& b) { v = v + b.v; d += b.d; return *this; }
    DualT& operator*=(const DualT& b) { d = d * double(b.v) + double(v) * b.d; v = v * b.v; return *this; }
};
template <class V> inline DualT<V> mk(V v, double d) { return DualT<V>(v, d, 0); }
template <class V> inline DualT<V> operator+(DualT<V> a, DualT<V> b) { return mk<V>(a.v + b.v, a.d + b.d); }
template <class V> inline DualT<V> operator-(DualT<V> a, DualT<V> b) { return mk<V>(a.v - b.v, a.d - b.d); }
template <class V> inline DualT<V> operator-(DualT<V> a) { return mk<V>(-a.v, -a.d); }
template <class V> inline DualT<V> operator*(DualT<V> a, DualT<V> b) {
    return mk<V>(a.v * b.v, a.d * double(b.v) + double(a.v) * b.d);
}
template <class V> inline DualT<V> operator/(DualT<V> a, DualT<V> b) {
    const double bv = double(b.v);
    return mk<V>(a.v / b.v, (a.d * bv - double(a.v) * b.d) / (bv * bv));
}
template <class V> inline bool operator<(DualT<V> a, DualT<V> b) { return a.v < b.v; }
template <class V> inline bool operator>(DualT<V> a, DualT<V> b) { return a.v > b.v; }
template <class V> inline bool operator<=(DualT<V> a, DualT<V> b) { return a.v <= b.v; }
template <class V> inline bool operator>=(DualT<V> a, DualT<V> b) { return a.v >= b.v; }
template <class V> inline bool operator==(DualT<V> a, DualT<V> b) { return a.v == b.v; }
template <class V> inline bool operator!=(DualT<V> a, DualT<V> b) { return a.v != b.v; }
template <class V> inline DualT<V> fma_r(DualT<V> a, DualT<V> b, DualT<V> c) {
    return mk<V>(fma_r(a.v, b.v, c.v), a.d * double(b.v) + double(a.v) * b.d + c.d);
}
template <class V> inline DualT<V> floor_r(DualT<V> a) { return mk<V>(floor_r(a.v), 0.0); }
template <class V> inline DualT<V> sqrt_r(DualT<V> a) {
    const V r = sqrt_r(a.v);
    return mk<V>(r, r > V(0) ? a.d / (2.0 * double(r)) : 0.0);
}
template <class V> inline bool isfinite_r(DualT<V> a) { return isfinite_r(a.v); }
template <class V> inline DualT<V> fabs_r(DualT<V> a) { return a.v < V(0) ? -a : a; }
template <class V> inline DualT<V> copysign_r(DualT<V> mag, DualT<V> sgn) {
    return std::signbit(mag.v) != std::signbit(sgn.v) ? -mag : mag;
}
// s_corr's power: the exponent is a parameter (no derivative taken).
template <class V> inline DualT<V> pow_r(DualT<V> a, DualT<V> b) {
    const double av = double(a.v), bv = double(b.v);
    const double dp = (av != 0.0) ? bv * std::pow(av, bv - 1.0) : (bv == 1.0 ? 1.0 : 0.0);
    return mk<V>(pow_r(a.v, b.v), dp * a.d);
}

// Parameters of the dual step: the FP64 oracle's (kernel constants recomputed
// in double) or the FP32 oracle's, with the direction's component along
// xsph_c.
template <class V>
P<DualT<V>> make_p_dual(const pbf_device_params& d, double dxsph_c) {
    using D = DualT<V>;
    P<V> q;
    if constexpr (sizeof(V) == 8)
        q = make_p64(d);
    else
        q = make_p<float>(d);
    P<D> p{};
    auto c = [](V x) { return mk<V>(x, 0.0); };
    p.h = c(q.h); p.h2 = c(q.h2); p.poly6 = c(q.poly6); p.spiky = c(q.spiky);
    p.mins = {c(q.mins.x), c(q.mins.y), c(q.mins.z)};
    p.maxs = {c(q.maxs.x), c(q.maxs.y), c(q.maxs.z)};
    p.cs = c(q.cs);
    p.dimx = q.dimx; p.dimy = q.dimy; p.dimz = q.dimz;
    p.g = {c(q.g.x), c(q.g.y), c(q.g.z)};
    p.rest = c(q.rest); p.dt = c(q.dt); p.inv_dt = c(q.inv_dt); p.e = c(q.e); p.mass = c(q.mass);
    p.xsph_c = mk<V>(q.xsph_c, dxsph_c);
    p.maxNeighbors = q.maxNeighbors;
    p.scorr_enable = q.scorr_enable;
    p.scorr_k = c(q.scorr_k); p.scorr_n = c(q.scorr_n); p.scorr_dq_h = c(q.scorr_dq_h); p.wq_min = c(q.wq_min);
    p.scorr_min = c(q.scorr_min); p.grad_r_eps = c(q.grad_r_eps); p.lambda_denom_eps = c(q.lambda_denom_eps);
    p.compliance = c(q.compliance);
    p.enable_lambda_clamp = q.enable_lambda_clamp;
    p.lambda_max_abs = c(q.lambda_max_abs);
    p.enable_disp_clamp = q.enable_disp_clamp;
    p.disp_clamp_max_h = c(q.disp_clamp_max_h);
    p.enable_relax = q.enable_relax;
    p.relax_omega = c(q.relax_omega);
    p.xsph_gate_enable = q.xsph_gate_enable; p.xsph_n_min = q.xsph_n_min; p.xsph_n_max = q.xsph_n_max;
    return p;
}

template <class V>
int step_jvp(const pbf_sim_params& sp, int hashed, double* pos4, double* vel4, double* dpos4, double* dvel4,
             double dxsph_c, uint32_t N, int steps) {
    using D = DualT<V>;
    const pbf_device_params dp = device_params_of(sp);
    const P<D> pd = make_p_dual<V>(dp, dxsph_c);
    std::vector<V4<D>> pos(N), vel(N);
    for (size_t i = 0; i < N; ++i)
        for (int c = 0; c < 4; ++c) {
            (&pos[i].x)[c] = mk<V>(V(pos4[4 * i + c]), dpos4[4 * i + c]);
            (&vel[i].x)[c] = mk<V>(V(vel4[4 * i + c]), dvel4[4 * i + c]);
        }
    for (int k = 0; k < steps; ++k) {
        const int rc = step_t<D>(sp, hashed, pos.data(), vel.data(), N, nullptr, pd);
        if (rc != 0) return rc;
    }
    for (size_t i = 0; i < N; ++i)
        for (int c = 0; c < 4; ++c) {
            pos4[4 * i + c] = double((&pos[i].x)[c].v);
            dpos4[4 * i + c] = (&pos[i].x)[c].d;
            vel4[4 * i + c] = double((&vel[i].x)[c].v);
            dvel4[4 * i + c] = (&vel[i].x)[c].d;
        }
    return 0;
}

}  // namespace

extern "C" {

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void oracle_integrate_pred(const float4* pos, const float4* vel, float4* pred, float3 g, float dt, uint32_t N) {
    integrate_pred_t<float>(as4(pos), as4(vel), as4(pred), V3<float>{g.x, g.y, g.z}, dt, N);
}

void oracle_boundary(float4* pred, float4* vel, const pbf_grid_bounds* g, float restitution, uint32_t N) {
    boundary_t<float>(as4(pred), as4(vel), V3<float>{g->mins.x, g->mins.y, g->mins.z},
                      V3<float>{g->maxs.x, g->maxs.y, g->maxs.z}, restitution, N);
}

void oracle_velocity(float4* vel, const float4* pos, const float4* pred, float inv_dt, uint32_t N) {
    velocity_t<float>(as4(vel), as4(pos), as4(pred), inv_dt, N);
}

void oracle_hash_keys(uint32_t* keys, uint32_t* indices, const float4* pred, const pbf_grid_bounds* g, uint32_t N) {
    hash_keys_t<float>(keys, indices, as4(pred), V3<float>{g->mins.x, g->mins.y, g->mins.z}, g->cellSize,
                       g->dim.x, g->dim.y, g->dim.z, N);
}

void oracle_sort_pairs(const uint32_t* kin, uint32_t* kout, const uint32_t* vin, uint32_t* vout, uint32_t N) {
    sort_pairs_impl(kin, kout, vin, vout, N);
}

void oracle_cell_ranges(uint32_t* start, uint32_t* end, const uint32_t* ks, uint32_t N, uint32_t numCells) {
    cell_ranges_impl(start, end, ks, N, numCells);
}

void oracle_cell_ranges_compact(uint32_t* uk, uint32_t* off, uint32_t* count, const uint32_t* ks, uint32_t N) {
    cell_compact_impl(uk, off, count, ks, N);
}

void oracle_lambda(float* lambda, const float4* pred, const uint32_t* idx, const uint32_t* keys,
                   const oracle_table* t, const pbf_device_params* dp, uint32_t N) {
    lambda_t<float>(lambda, as4(pred), idx, keys, make_table(t), make_p<float>(*dp), N);
}

void oracle_delta_apply(float4* pred, float4* delta, const float* lambda, const uint32_t* idx,
                        const uint32_t* keys, const oracle_table* t, const pbf_device_params* dp, uint32_t N) {
    delta_apply_t<float>(as4(pred), as4(delta), lambda, idx, keys, make_table(t), make_p<float>(*dp), N);
}

void oracle_xsph(float4* vel_out, const float4* vel_in, const float4* pred, const uint32_t* idx,
                 const uint32_t* keys, const oracle_table* t, const pbf_device_params* dp, uint32_t N) {
    xsph_t<float>(as4(vel_out), as4(vel_in), as4(pred), idx, keys, make_table(t), make_p<float>(*dp), N);
}

int oracle_step_f32(const pbf_sim_params* p, int hashed, float4* pos, float4* vel, uint32_t N,
                    oracle_trace* trace) {
    pbf_sim_params sp = *p;
    compute_dims(sp.grid);
    pbf_device_params dp = device_params_of(sp);
    return step_t<float>(sp, hashed, as4(pos), as4(vel), N, trace, make_p<float>(dp));
}

int oracle_step_f64(const pbf_sim_params* p, int hashed, double* pos4, double* vel4, uint32_t N) {
    pbf_sim_params sp = *p;
    compute_dims(sp.grid);
    pbf_device_params dp = device_params_of(sp);
    return step_t<double>(sp, hashed, reinterpret_cast<V4<double>*>(pos4), reinterpret_cast<V4<double>*>(vel4),
                          N, nullptr, make_p64(dp));
}

void oracle_density_stats_f32pos(const pbf_sim_params* p, const float4* pos, uint32_t N, double out[4]) {
    std::vector<double> x(4 * size_t(N));
    for (uint32_t i = 0; i < N; ++i) {
        x[4 * i] = pos[i].x;
        x[4 * i + 1] = pos[i].y;
        x[4 * i + 2] = pos[i].z;
        x[4 * i + 3] = 1.0;
    }
    density_stats_impl(*p, x.data(), N, out);
}

void oracle_density_stats_f64pos(const pbf_sim_params* p, const double* pos4, uint32_t N, double out[4]) {
    density_stats_impl(*p, pos4, N, out);
}

int oracle_step_jvp(const pbf_sim_params* p, int hashed, int fp32_values, double* pos4, double* vel4,
                    double* dpos4, double* dvel4, double dxsph_c, uint32_t N, int steps) {
    pbf_sim_params sp = *p;
    compute_dims(sp.grid);
    return fp32_values ? step_jvp<float>(sp, hashed, pos4, vel4, dpos4, dvel4, dxsph_c, N, steps)
                       : step_jvp<double>(sp, hashed, pos4, vel4, dpos4, dvel4, dxsph_c, N, steps);
}

int oracle_dam_break_params(float bx, float by, float bz, int solver_iters, uint32_t num_particles,
                            pbf_sim_params* out) {
    if (!out || !(bx > 0.f) || !(by > 0.f) || !(bz > 0.f) || solver_iters < 0) return 1;
    pbf_sim_params sp;
    std::memset(&sp, 0, sizeof(sp));
    const float r = 0.005f, spacing = 0.01f, h = 2.5f * r;
    sp.numParticles = sp.maxParticles = num_particles;
    sp.gravity.x = 0.f;
    sp.gravity.y = -9.8f;
    sp.gravity.z = 0.f;
    sp.dt = 1.0f / 120.0f;
    sp.cfl = 0.45f;
    sp.solverIters = solver_iters;
    sp.maxNeighbors = 64;
    sp.sortEveryN = 1;
    sp.boundaryRestitution = 0.f;
    sp.particleMass = 1000.0f * spacing * spacing * spacing;
    // tuning: sim/parameters.h:28-56 defaults, then the dam-break values
    pbf_tuning& t = sp.pbf;
    t.scorr_enable = 1;
    t.scorr_k = 0.1f;
    t.scorr_n = 4.0f;
    t.scorr_dq_h = 0.2f;
    t.wq_min = 1e-12f;
    t.scorr_min = -0.25f;
    t.grad_r_eps = 1e-6f;
    t.lambda_denom_eps = 100.0f;
    t.compliance = 0.f;
    t.xpbd_enable = 0;
    t.enable_lambda_clamp = 1;
    t.lambda_max_abs = 50.0f;
    t.enable_disp_clamp = 1;
    t.disp_clamp_max_h = 0.05f;
    t.enable_relax = 1;
    t.relax_omega = 0.75f;
    t.xsph_gate_enable = 0;
    t.xsph_n_min = 0;
    t.xsph_n_max = 8;
    t.lambda_warm_start_enable = 0;
    t.lambda_warm_start_decay = 0.5f;
    t.semi_implicit_integration_enable = 0;
    sp.xsph_c = 0.01f;
    // kernel coefficients, sim/parameters.h:94-107 (FP32, same operation order)
    pbf_kernel_coeffs& kc = sp.kernel;
    const float pi = 3.14159265358979323846f;
    kc.h = h;
    kc.inv_h = 1.0f / h;
    kc.h2 = h * h;
    const float h3 = h * kc.h2, h6 = h3 * h3, h9 = h6 * h3;
    kc.poly6 = 315.0f / (64.0f * pi * h9);
    kc.spiky = 15.0f / (pi * h6);
    kc.visc = 15.0f / (2.0f * pi * h3);
    float density = 0.f;
    for (int n = 0; n < 6; ++n) {
        const float r2 = spacing * spacing;
        const float hr2 = kc.h2 - r2;
        density += sp.particleMass * kc.poly6 * hr2 * hr2 * hr2;
    }
    sp.restDensity = density;
    sp.grid.mins.x = sp.grid.mins.y = sp.grid.mins.z = 0.f;
    sp.grid.maxs.x = bx;
    sp.grid.maxs.y = by;
    sp.grid.maxs.z = bz;
    sp.grid.cellSize = std::fmax(1e-6f, 1.0f * h);
    compute_dims(sp.grid);
    sp.grid.dim.x = std::max(sp.grid.dim.x, 1);
    sp.grid.dim.y = std::max(sp.grid.dim.y, 1);
    sp.grid.dim.z = std::max(sp.grid.dim.z, 1);
    *out = sp;
    return 0;
}

void oracle_seed_lattice(float4* out, uint32_t nx, uint32_t ny, uint32_t nz, float ox, float oy, float oz,
                         float spacing, float jitter, uint64_t seed, const pbf_grid_bounds* box) {
    std::mt19937_64 rng(seed);
    auto unit = [&]() { return double(rng() >> 11) * (1.0 / 9007199254740992.0); };
    const pbf_grid_bounds& g = *box;
    size_t id = 0;
    for (uint32_t iz = 0; iz < nz; ++iz)
        for (uint32_t iy = 0; iy < ny; ++iy)
            for (uint32_t ix = 0; ix < nx; ++ix) {
                const float jx = float((2.0 * unit() - 1.0) * double(jitter));
                const float jy = float((2.0 * unit() - 1.0) * double(jitter));
                const float jz = float((2.0 * unit() - 1.0) * double(jitter));
                out[id].x = std::fmin(std::fmax(ox + float(ix) * spacing + jx, g.mins.x), g.maxs.x);
                out[id].y = std::fmin(std::fmax(oy + float(iy) * spacing + jy, g.mins.y), g.maxs.y);
                out[id].z = std::fmin(std::fmax(oz + float(iz) * spacing + jz, g.mins.z), g.maxs.z);
                out[id].w = 1.0f;
                ++id;
            }
}

}  // extern "C"
