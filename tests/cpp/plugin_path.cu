// plugin_path.cu - the C++ half of the drop-in boundary, exercised.
//
// A program written against include/pbf/simulator.h (sim::Simulator and the
// KernelDispatcher plugin API of sim/kernel_dispatcher.h:14-36) registers its
// own launcher for PhaseType::Post and checks that it replaced the built-in
// one.  The user launcher commits the solved prediction and the velocities
// without XSPH (a "Post without XSPH" plugin).  So a scene with XSPH on,
// stepped with the user launcher, must give the same bits as the same scene
// with XSPH off stepped with the built-in launchers, and must differ from
// the scene with XSPH on stepped with the built-in launchers.
//
// Built by __graft_entry__.build() against libpbf_gb300.so; run by
// tests/test_gpu_plugin_path.py.  Prints "PLUGIN OK ..." and exits 0 on
// success.
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/pbf/pbf.h"
#include "../../include/pbf/simulator.h"

namespace {

int g_userPostCalls = 0;

__global__ void k_user_post(const float4* __restrict__ pred_s, const float4* __restrict__ vel_s,
                            const uint32_t* __restrict__ perm, uint32_t n, float4* __restrict__ pos,
                            float4* __restrict__ vel) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = perm[s];  // sorted slot -> particle id
    pos[i] = pred_s[s];
    vel[i] = vel_s[s];
}

// A KernelLaunchFn: the solved prediction and the velocity phase's output are
// in cell order; d_pos / d_vel are in particle order.
void UserPost(sim::DeviceBuffers& b, sim::GridBuffers& g, const sim::SimParams& p, cudaStream_t s) {
    ++g_userPostCalls;
    const uint32_t n = p.numParticles;
    k_user_post<<<(n + 255) / 256, 256, 0, s>>>(sim::SolvedPrediction(b, p.solverIters), b.d_vel_sorted,
                                                 g.d_indices_sorted, n, b.d_pos, b.d_vel);
}

sim::SimParams scene(float xsph_c) {
    pbf_sim_params c{};
    if (pbf_dam_break_params(0.4f, 0.4f, 0.4f, 2, 16 * 16 * 16, &c) != PBF_OK) std::abort();
    sim::SimParams p;
    std::memcpy(&p, &c, sizeof(p));
    p.xsph_c = xsph_c;
    return p;
}

struct Run {
    std::vector<float4> pos, vel;
};

Run run(float xsph_c, bool userPost, int steps) {
    sim::Simulator s;
    const sim::SimParams p = scene(xsph_c);
    if (!s.initialize(p, true)) std::abort();
    s.seedBoxLattice(16, 16, 16, make_float3(0.005f, 0.005f, 0.005f), 0.01f);
    if (userPost) {
        // the variant the hashed pipeline looks up (compact = true); the
        // lookup falls back from halfVel / halfPos to this key
        s.dispatcher().registerKernel(sim::PhaseType::Post, false, false, true, UserPost);
        s.invalidateGraph();
    }
    for (int k = 0; k < steps; ++k)
        if (!s.step(p)) std::abort();
    Run r;
    r.pos.resize(p.numParticles);
    r.vel.resize(p.numParticles);
    if (cudaStreamSynchronize(s.cudaStream()) != cudaSuccess ||
        cudaMemcpy(r.pos.data(), s.devicePositions(), sizeof(float4) * p.numParticles, cudaMemcpyDeviceToHost) !=
            cudaSuccess ||
        cudaMemcpy(r.vel.data(), s.deviceVel(), sizeof(float4) * p.numParticles, cudaMemcpyDeviceToHost) !=
            cudaSuccess)
        std::abort();
    if (s.takeDeviceError() != 0) std::abort();
    return r;
}

bool same(const Run& a, const Run& b) {
    return std::memcmp(a.pos.data(), b.pos.data(), sizeof(float4) * a.pos.size()) == 0 &&
           std::memcmp(a.vel.data(), b.vel.data(), sizeof(float4) * a.vel.size()) == 0;
}

}  // namespace

int main() {
    const int steps = 5;
    const Run noXsph = run(0.0f, false, steps);
    const Run builtIn = run(0.01f, false, steps);
    const Run plugin = run(0.01f, true, steps);
    if (g_userPostCalls != 1) {
        std::printf("FAIL: user launcher called %d times (expected once, at graph capture)\n", g_userPostCalls);
        return 1;
    }
    if (!same(plugin, noXsph)) {
        std::printf("FAIL: the user Post launcher's run differs from the built-in run without XSPH\n");
        return 1;
    }
    if (same(plugin, builtIn)) {
        std::printf("FAIL: the built-in Post (with XSPH) gives the same state: the user launcher made no difference\n");
        return 1;
    }
    std::printf("PLUGIN OK calls=%d particles=%zu steps=%d\n", g_userPostCalls, plugin.pos.size(), steps);
    return 0;
}
