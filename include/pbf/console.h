// console.h - headless runtime configuration of PBF-X: console::RuntimeConsole
// and the mapping from it to sim::SimParams.
//
// Source-compatible with the simulation-relevant part of the reference's
// engine/core/console.h:122-243 (RuntimeConsole::Simulation and ::Performance:
// same field names, types and defaults) and with its mapping functions:
//   BuildSimParams     engine/core/console.cpp:198-265
//   PrepareCubeMix     engine/core/console.cpp:360-386 (CubeMix layout and
//                      domain, engine/core/console.cpp:55-182)
//   SanitizeSimParams  the parameter clamps of app_main.cpp:454-496
//   MergeConfigJson    config::LoadFile's merge of config.json,
//                      engine/core/config.cpp:160-238 and :331-342
// Window, viewer, camera, colour, debug and benchmark settings are renderer or
// application state and are not part of this header.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "parameters.h"

namespace console {

struct RuntimeConsole {
    struct Simulation {
        Simulation();
        void refreshCubeMixDerived();

        uint32_t numParticles = 800000;
        uint32_t maxParticles = 10000000;

        float dt = 0.016667f;
        float cfl = 0.45f;

        float3 gravity = make_float3(0.0f, -9.8f, 0.0f);
        float restDensity = 1.0f;

        enum class MassMode : uint32_t { Explicit = 0, SphereByRadius = 1, UniformLattice = 2 };
        MassMode massMode = MassMode::UniformLattice;
        float lattice_spacing_factor_h = 1.0f;
        float particleMass = 1.0f;
        float particleVolumeScale = 1.0f;

        float particleRadiusWorld = 1.0f;
        bool deriveHFromRadius = true;
        float h_over_r = 2.5f;

        sim::PbfTuning pbf{};
        float xsph_c = 0.05f;

        float smoothingRadius = 3.5f;
        float3 gridMins = make_float3(0.0f, 0.0f, 0.0f);
        float3 gridMaxs = make_float3(200.0f, 200.0f, 200.0f);
        float cellSize = 0.0f;

        int solverIters = 1;
        int maxNeighbors = 64;
        float boundaryRestitution = 0.0f;

        enum class DemoMode : uint32_t { CubeMix = 1 };
        DemoMode demoMode = DemoMode::CubeMix;

        bool cube_auto_partition = false;
        uint32_t cube_group_count = 8;
        uint32_t cube_edge_particles = 60;
        static constexpr uint32_t cube_group_count_max = 512;
        uint32_t cube_layers = 2;
        float cube_group_spacing_world = 200.0f;
        float cube_layer_spacing_world = 200.0f;
        float cube_base_height = 200.0f;
        float cube_lattice_spacing_factor_h = 1.02f;
        float cube_initial_density = 1.0f;
        bool cube_auto_fit_domain = true;
        float cube_domain_margin_scale = 1.2f;
        bool cube_apply_initial_jitter = true;
        bool cube_layer_jitter_enable = false;
        float cube_layer_jitter_scale_h = 0.05f;
        uint32_t cube_layer_jitter_seed = 0x13579BDFu;
        uint32_t cube_particles_per_group = 0;

        bool integrate_semi_implicit = true;
        bool lambda_warm_start_enable = true;
        float lambda_warm_start_decay = 0.5f;
        bool xpbd_enable = true;
        float xpbd_compliance = 2e-5f;

        bool initial_jitter_enable = true;
        float initial_jitter_scale_h = 0.01f;
        uint32_t initial_jitter_seed = 0xC0FFEEu;
    } sim;

    struct Performance {
        float grid_cell_size_multiplier = 1.0f;
        int neighbor_cap = 0;
        int launch_bounds_tbs = 256;
        int min_blocks_per_sm = 2;
        bool use_hashed_grid = false;
        int sort_compact_every_n = 1;
        bool compact_binary_search = true;
        bool log_grid_compact_stats = false;
    } perf;
};

// CubeMix scene: group count (clamped to [1, cube_group_count_max]), particles
// per group and total (numParticles), the split of groups over layers and,
// with cube_auto_fit_domain, the simulation box around them.  The group
// colours of the reference are renderer state and are not computed.
void PrepareCubeMix(RuntimeConsole& c);

// The CubeMix group centres the seeding places its cubes on, layer by layer
// (engine/core/console.cpp:276-314).
void GenerateCubeMixCenters(const RuntimeConsole& c, std::vector<float3>& outCenters);

// sim::SimParams for the console: fields not written here keep their values
// in `out` (the reference starts from SimParams{}).
void BuildSimParams(const RuntimeConsole& c, sim::SimParams& out);
void BuildDeviceParams(const RuntimeConsole& c, sim::DeviceParams& out);

// The reference application's guard rails on the parameters: solverIters in
// [1, 64], maxNeighbors in [8, perf.neighbor_cap when > 0, else 1024],
// sortEveryN >= 1.
void SanitizeSimParams(const RuntimeConsole& c, sim::SimParams& sp);

// Merges a config.json text: "performance" and "simulation" keys, the
// "profile" name and that profile's overrides, then PrepareCubeMix.  Returns
// false with *err set, and the console unchanged, when the text is not JSON
// or a known key has a value of the wrong type.  *activeProfile (may be null)
// receives the profile named by the text, if any.
bool MergeConfigJson(RuntimeConsole& c, const std::string& text, std::string* activeProfile, std::string* err);

}  // namespace console
