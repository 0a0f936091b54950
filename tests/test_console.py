"""Runtime configuration: the reference application's RuntimeConsole defaults,
CubeMix derivation, config.json merge and RuntimeConsole -> SimParams mapping
(engine/core/console.h:122-243, engine/core/console.cpp:55-386,
engine/core/config.cpp:160-342, app_main.cpp:454-496).

The reference's console code does not build here (it includes the D3D12
renderer), so the expected values are restated below from its formulas in
float32, operation by operation, and compared bit for bit.  Host code only:
no GPU.
"""
import math

import numpy as np
import pytest

import pbfx

f32 = np.float32


@pytest.fixture()
def con(lib):
    c = pbfx.Console(lib)
    yield c
    c.close()


def cube_mix_expected(groups=8, edge=60, layers=2, kernel_radius=3.5, lattice=1.02, spacing_world=200.0,
                      layer_spacing=200.0, base=200.0, margin=1.2):
    """(centres, grid mins, grid maxs) of the CubeMix scene, console.cpp:55-182."""
    per_layer, remaining = [], groups
    for L in range(layers):
        take = max(1, remaining // (layers - L))
        per_layer.append(take)
        remaining -= take
    h = f32(kernel_radius) if f32(kernel_radius) > f32(1e-6) else f32(1e-6)
    spacing = h * f32(lattice)
    half = (spacing * f32(edge)) * f32(0.5)
    lo = [f32(1e30)] * 3
    hi = [f32(-1e30)] * 3
    centres = []
    for layer, n in enumerate(per_layer):
        nx = math.ceil(math.sqrt(n))
        y = f32(base) + f32(layer) * f32(layer_spacing)
        for k in range(n):
            c = [f32(k % nx) * f32(spacing_world), y, f32(k // nx) * f32(spacing_world)]
            centres.append(c)
            lo = [min(lo[a], c[a] - half) for a in range(3)]
            hi = [max(hi[a], c[a] + half) for a in range(3)]
    size = [hi[a] - lo[a] for a in range(3)]
    mn = [lo[0], min(f32(0), lo[1] - half), lo[2]]
    mx = [lo[a] + size[a] for a in range(3)]
    centre = [(mn[a] + mx[a]) * f32(0.5) for a in range(3)]
    hh = [(mx[a] - mn[a]) * f32(0.5) * f32(margin) for a in range(3)]
    gmin = [centre[0] - hh[0], max(f32(0), centre[1] - hh[1]), centre[2] - hh[2]]
    gmax = [centre[a] + hh[a] for a in range(3)]
    return np.array(centres, np.float32), gmin, gmax


def test_defaults_are_the_reference_console(con):
    assert con["sim.numParticles"] == 8 * 60 ** 3
    assert con["sim.cube_particles_per_group"] == 60 ** 3
    centres, gmin, gmax = cube_mix_expected()
    for a, ax in enumerate("xyz"):
        assert f32(con["sim.gridMins." + ax]) == gmin[a]
        assert f32(con["sim.gridMaxs." + ax]) == gmax[a]
    np.testing.assert_array_equal(con.cube_mix_centers(), centres)
    # a sample of the other defaults
    assert f32(con["sim.dt"]) == f32(0.016667) and f32(con["sim.xpbd_compliance"]) == f32(2e-5)
    assert con["sim.massMode"] == 2 and con["sim.deriveHFromRadius"] == 1 and con["perf.use_hashed_grid"] == 0
    assert f32(con["sim.pbf.scorr_k"]) == f32(0.003) and con["perf.launch_bounds_tbs"] == 256


def test_sim_params_of_the_defaults(con):
    p = con.sim_params(sanitize=False)
    h = f32(2.5) * f32(1.0)  # h_over_r * particleRadiusWorld
    assert f32(p.kernel.h) == h
    assert f32(p.particleMass) == f32(1.0) * h * h * h  # uniform lattice, factor 1
    assert f32(p.grid.cellSize) == h
    _, gmin, gmax = cube_mix_expected()
    dims = [max(1, int(math.ceil(f32(gmax[a] - gmin[a]) / h))) for a in range(3)]
    assert (p.grid.dim.x, p.grid.dim.y, p.grid.dim.z) == tuple(dims)
    assert p.numParticles == 1728000 and p.maxParticles == 10000000
    assert p.solverIters == 1 and p.maxNeighbors == 64 and f32(p.xsph_c) == f32(0.05)
    # the console's stability switches override the tuning block
    assert p.pbf.xpbd_enable == 1 and f32(p.pbf.compliance) == f32(2e-5)
    assert p.pbf.lambda_warm_start_enable == 1 and p.pbf.semi_implicit_integration_enable == 1
    assert p.sortEveryN == 0  # not written by BuildSimParams
    assert con.sim_params().sortEveryN == 1  # the application's clamp


def test_smoothing_length_and_mass_modes(con):
    con["sim.particleRadiusWorld"] = 0.005
    con["sim.restDensity"] = 1000.0
    r = f32(0.005)
    h = f32(2.5) * r
    p = con.sim_params()
    assert f32(p.kernel.h) == h
    assert f32(p.particleMass) == f32(1000.0) * h * h * h
    con["sim.lattice_spacing_factor_h"] = 0.8
    spacing = f32(0.8) * h
    assert f32(con.sim_params().particleMass) == f32(1000.0) * spacing * spacing * spacing
    con["sim.massMode"] = 1  # sphere by radius
    con["sim.particleVolumeScale"] = 1.5
    pi = f32(math.pi)
    vol = f32(1.5) * (f32(4.0) / f32(3.0)) * pi * r * r * r
    assert f32(con.sim_params().particleMass) == vol * f32(1000.0)
    con["sim.massMode"] = 0  # explicit
    con["sim.particleMass"] = 0.125
    assert f32(con.sim_params().particleMass) == f32(0.125)
    with pytest.raises(RuntimeError):
        con["sim.massMode"] = 3
    # h from the kernel radius, or 0.02 without one
    con["sim.deriveHFromRadius"] = 0
    assert f32(con.sim_params().kernel.h) == f32(3.5)
    con["sim.smoothingRadius"] = 0.0
    assert f32(con.sim_params().kernel.h) == f32(0.02)


def test_cell_size_and_neighbour_cap(con):
    con["perf.grid_cell_size_multiplier"] = 2.0
    assert f32(con.sim_params().grid.cellSize) == f32(2.0) * f32(2.5)
    con["perf.grid_cell_size_multiplier"] = -1.0  # not positive: 1
    assert f32(con.sim_params().grid.cellSize) == f32(2.5)
    con["sim.cellSize"] = 4.0
    p = con.sim_params()
    assert f32(p.grid.cellSize) == f32(4.0)
    ext = f32(con["sim.gridMaxs.y"]) - f32(con["sim.gridMins.y"])
    assert p.grid.dim.y == max(1, math.ceil(ext / f32(4.0)))
    con["perf.neighbor_cap"] = 32
    assert con.sim_params().maxNeighbors == 32
    con["perf.neighbor_cap"] = 0
    con["sim.xpbd_enable"] = 0
    p = con.sim_params()
    assert p.pbf.xpbd_enable == 0 and p.pbf.compliance == 0.0


def test_application_clamps(con):
    for iters, want in ((0, 1), (-3, 1), (7, 7), (100, 64)):
        con["sim.solverIters"] = iters
        assert con.sim_params().solverIters == want
        assert con.sim_params(sanitize=False).solverIters == iters
    for mn, cap, want in ((4, 0, 8), (5000, 0, 1024), (200, 96, 96), (64, 0, 64)):
        con["sim.maxNeighbors"] = mn
        con["perf.neighbor_cap"] = cap
        assert con.sim_params().maxNeighbors == want


def test_merge_config_json(con):
    text = """{
      "system": {"resolution": [1920, 1080], "vsync": false},
      "viewer": {"enabled": true, "point_size_px": 3},
      "performance": {"grid_cell_size_multiplier": 1.5, "neighbor_cap": 48, "use_hashed_grid": true,
                      "sort_compact_every_n": 2, "unknown_key": [1, 2, {"a": null}]},
      "simulation": {"cfl": 0.3, "rest_density": 1000, "kernel_radius": 0.05, "solver_iterations": 3.9,
                     "max_neighbors": 96, "xsph_c": 0.02, "xsph_c": 0.03},
      "profile": "fast",
      "profiles": {"fast": {"simulation": {"solver_iterations": 2}, "performance": {"neighbor_cap": 40}},
                   "slow": {"simulation": {"solver_iterations": 8}}}
    }"""
    con.merge_json(text)
    assert f32(con["perf.grid_cell_size_multiplier"]) == f32(1.5)
    assert con["perf.use_hashed_grid"] == 1 and con["perf.sort_compact_every_n"] == 2
    assert f32(con["sim.cfl"]) == f32(0.3) and f32(con["sim.restDensity"]) == f32(1000.0)
    assert f32(con["sim.smoothingRadius"]) == f32(0.05)
    assert f32(con["sim.xsph_c"]) == f32(0.03)  # the last of duplicate keys
    assert con["sim.maxNeighbors"] == 96
    assert con.profile() == "fast"
    assert con["sim.solverIters"] == 2 and con["perf.neighbor_cap"] == 40  # the profile's overrides
    p = con.sim_params()
    assert p.maxNeighbors == 40 and p.solverIters == 2
    # the CubeMix scene is re-derived from the new kernel radius
    _, gmin, gmax = cube_mix_expected(kernel_radius=0.05)
    assert f32(con["sim.gridMaxs.x"]) == gmax[0] and f32(con["sim.gridMins.z"]) == gmin[2]
    # a later text without a profile key keeps applying the active profile
    con.merge_json('{"simulation": {"solver_iterations": 5}, "profiles": {"fast": {"simulation": '
                   '{"solver_iterations": 6}}}}')
    assert con["sim.solverIters"] == 6 and con.profile() == "fast"
    # solver_iterations 3.9 would have been read as 3 without the profile
    con.merge_json('{"profile": "none", "simulation": {"solver_iterations": 3.9}}')
    assert con["sim.solverIters"] == 3


@pytest.mark.parametrize("text", ["{", '{"performance": {"use_hashed_grid": 1}}', '{"simulation": {"cfl": "0.3"}}',
                                  '{"a": 1} x', '{"profile": "p", "profiles": {"p": {"simulation": '
                                  '{"max_neighbors": true}}}}', "[1, 2", '{"a": "\\q"}', "", "nul"])
def test_rejected_config_leaves_the_console_unchanged(con, text):
    before = (con["sim.cfl"], con["sim.maxNeighbors"], con["perf.use_hashed_grid"], con.profile())
    with pytest.raises(ValueError):
        con.merge_json(text)
    assert (con["sim.cfl"], con["sim.maxNeighbors"], con["perf.use_hashed_grid"], con.profile()) == before


def test_json_corner_cases_accepted(con):
    con.merge_json('  {"simulation": {"cfl": 25e-2, "xsph_c": -0.0, "max_neighbors": -7}, '
                   '"note": "caf\\u00e9 \\ud83d\\ude00 \\"q\\" \\\\", "list": [], "o": {}}  ')
    assert f32(con["sim.cfl"]) == f32(0.25) and con["sim.maxNeighbors"] == -7
    assert con.sim_params().maxNeighbors == 8
    con.merge_json('"not an object"')  # no known section: nothing changes
    assert f32(con["sim.cfl"]) == f32(0.25)


def auto_partition(target, gmax=512):
    target = max(1, target)
    L = max(1, round(target ** (1.0 / 3.0)))
    G = max(1, target // L ** 3)
    while G * L ** 3 > target and L > 1:
        L -= 1
    while G * (L + 1) ** 3 <= target:
        L += 1
    while (G + 1) * L ** 3 <= target and G + 1 <= gmax:
        G += 1
    return L, min(G, gmax)


@pytest.mark.parametrize("target", [1, 27, 1000000, 2000000, 3000000, 12345678, 700000])
def test_cube_mix_auto_partition(con, target):
    con["sim.cube_auto_partition"] = 1
    con["sim.numParticles"] = target
    con.prepare_cube_mix()
    L, G = auto_partition(target)
    assert con["sim.cube_edge_particles"] == L and con["sim.cube_group_count"] == G
    assert con["sim.numParticles"] == (G * L ** 3) % 2 ** 32
    assert con["sim.numParticles"] <= target


def test_cube_mix_groups_and_layers(con):
    con["sim.cube_group_count"] = 7
    con["sim.cube_layers"] = 3
    con["sim.cube_edge_particles"] = 10
    con["sim.smoothingRadius"] = 0.05
    con.prepare_cube_mix()
    centres, gmin, gmax = cube_mix_expected(groups=7, edge=10, layers=3, kernel_radius=0.05)
    np.testing.assert_array_equal(con.cube_mix_centers(), centres)
    assert [f32(con["sim.gridMins." + a]) for a in "xyz"] == gmin
    assert [f32(con["sim.gridMaxs." + a]) for a in "xyz"] == gmax
    assert con["sim.numParticles"] == 7000
    con["sim.cube_group_count"] = 0  # clamped to one group
    con["sim.cube_layers"] = 5  # and to one layer per group
    con.prepare_cube_mix()
    assert con["sim.cube_group_count"] == 1 and con["sim.cube_layers"] == 1
    assert len(con.cube_mix_centers()) == 1


def test_unknown_field(con):
    with pytest.raises(RuntimeError):
        con["sim.no_such_field"] = 1
    with pytest.raises(RuntimeError):
        con["perf.neighbor_cap"] = 1e20


@pytest.mark.gpu
def test_seed_cube_mix(gpu, lib, con):
    """The application's CubeMix seeding through the console: group count x
    edge^3 particles, each group a lattice cube about its centre, inside the
    derived box."""
    con["sim.cube_group_count"] = 4
    con["sim.cube_edge_particles"] = 12
    con["sim.particleRadiusWorld"] = 0.005
    con["sim.smoothingRadius"] = 0.0125
    con["sim.cube_group_spacing_world"] = 0.5
    con["sim.cube_layer_spacing_world"] = 0.4
    con["sim.cube_base_height"] = 0.3
    con.prepare_cube_mix()
    p = con.sim_params()
    assert p.numParticles == 4 * 12 ** 3
    with pbfx.Sim(lib, p, hashed=False) as s:
        pbfx.check(lib.pbf_seed_cube_mix(s.h, con.h), "seed_cube_mix")
        pos, vel = s.download()
    assert pos.shape == (4 * 12 ** 3, 4) and np.all(vel[:, :3] == 0)
    lo = np.array([p.grid.mins.x, p.grid.mins.y, p.grid.mins.z], np.float32)
    hi = np.array([p.grid.maxs.x, p.grid.maxs.y, p.grid.maxs.z], np.float32)
    assert np.all(pos[:, :3] >= lo) and np.all(pos[:, :3] <= hi)
    centres = con.cube_mix_centers()
    side = p.kernel.h * 1.02 * 12
    for g in range(4):
        part = pos[g * 12 ** 3:(g + 1) * 12 ** 3, :3]
        assert np.all(np.abs(part.mean(axis=0) - centres[g]) < 0.1 * side)
