"""Batched ensemble vs the scenes stepped one by one.

Every scene of an ensemble must evolve bit-identically to a pbf_sim with the
same parameters and initial state: the batched step sorts by (scene, cell,
particle), which inside a scene is the scene's own (cell, particle) order,
and each particle reads only its scene's parameters and neighbours.
"""
import ctypes as C

import numpy as np
import pytest

import pbfx


def mixed_scenes(lib):
    scenes, pos = pbfx.ensemble_scenes(lib, 7, seed=11, n_min=300, n_max=6000, iters_choices=(0, 1, 2, 3))
    # vary what the step branches on: XSPH off, displacement clamp off (no
    # lists in the single-scene step), s_corr off, a neighbour cap
    scenes[1].xsph_c = 0.0
    scenes[2].pbf.enable_disp_clamp = 0
    scenes[3].pbf.scorr_enable = 0
    scenes[4].maxNeighbors = 12
    return scenes, pos


def step_alone(lib, p, pos, vel, steps):
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.upload(pos, vel)
        s.step(steps)
        return s.download()


@pytest.mark.gpu
def test_ensemble_matches_scenes_stepped_alone(gpu, lib):
    scenes, pos = mixed_scenes(lib)
    vel = np.zeros_like(pos)
    steps = 25
    with pbfx.Ensemble(lib, scenes) as e:
        off = e.offsets
        assert off[0] == 0 and off[-1] == pos.shape[0] == e.n
        e.upload(pos, vel)
        e.step(steps)
        epos, evel = e.download()
    assert np.all(np.isfinite(epos))
    for k, p in enumerate(scenes):
        a, b = int(off[k]), int(off[k + 1])
        assert b - a == p.numParticles
        spos, svel = step_alone(lib, p, pos[a:b], vel[a:b], steps)
        np.testing.assert_array_equal(epos[a:b], spos, err_msg="scene %d positions" % k)
        np.testing.assert_array_equal(evel[a:b], svel, err_msg="scene %d velocities" % k)


@pytest.mark.gpu
def test_ensemble_host_step_and_empty_scene(gpu, lib):
    scenes, pos = pbfx.ensemble_scenes(lib, 3, seed=5, n_min=1000, n_max=3000)
    empty = pbfx.dam_break_params((0.4, 0.4, 0.4), 2, 0)
    scenes.insert(1, empty)
    vel = np.zeros_like(pos)
    with pbfx.Ensemble(lib, scenes) as e:
        assert e.offsets[1] == e.offsets[2]
        hp, hv = pos.copy(), vel.copy()
        for _ in range(3):
            pbfx.check(lib.pbf_ensemble_step_host(e.h, pbfx.ptr(hp), pbfx.ptr(hv)))
        e.upload(pos, vel)
        e.step(3)
        dp, dv = e.download()
    np.testing.assert_array_equal(hp, dp)
    np.testing.assert_array_equal(hv, dv)


def test_ensemble_rejects_bad_arguments(lib):
    out = C.c_void_p()
    p = (pbfx.SimParams * 1)(pbfx.dam_break_params((0.5, 0.5, 0.5), 2, 100))
    assert lib.pbf_ensemble_create(p, 0, C.byref(out)) == pbfx.PBF_ERR_INVALID
    assert lib.pbf_ensemble_create(None, 1, C.byref(out)) == pbfx.PBF_ERR_INVALID
    assert lib.pbf_ensemble_create(p, 1, None) == pbfx.PBF_ERR_INVALID
    p[0].grid.cellSize = 0.0
    assert lib.pbf_ensemble_create(p, 1, C.byref(out)) == pbfx.PBF_ERR_INVALID
    assert not out.value
    assert lib.pbf_ensemble_step(None, 1) == pbfx.PBF_ERR_INVALID


def test_ensemble_scene_generator_is_seeded(lib):
    a, pa = pbfx.ensemble_scenes(lib, 4, seed=3)
    b, pb = pbfx.ensemble_scenes(lib, 4, seed=3)
    np.testing.assert_array_equal(pa, pb)
    assert [s.numParticles for s in a] == [s.numParticles for s in b]
    for s in a:
        # log-uniform in [2048, 65536], capped by what the box holds at spacing 0.01
        assert 2048 <= s.numParticles <= 65536 and s.solverIters in (2, 3)
        ext = (s.grid.maxs.x - s.grid.mins.x, s.grid.maxs.y - s.grid.mins.y, s.grid.maxs.z - s.grid.mins.z)
        assert all(0.3 <= e <= 1.0 + 1e-6 for e in ext)
        g = np.array([s.gravity.x, s.gravity.y, s.gravity.z])
        assert abs(np.linalg.norm(g) - 9.8) < 1e-4 and -g[1] / 9.8 >= np.cos(np.radians(15.0)) - 1e-6


@pytest.mark.gpu
def test_ensemble_caller_stream(gpu, lib):
    """pbf_ensemble_set_stream: the same state on a caller's stream."""
    torch = pytest.importorskip("torch")
    scenes, pos = mixed_scenes(lib)
    vel = np.zeros_like(pos)
    with pbfx.Ensemble(lib, scenes) as e:
        e.upload(pos, vel)
        e.step(8)
        ref = e.download()
    st = torch.cuda.Stream()
    with pbfx.Ensemble(lib, scenes) as e:
        own = e.stream_ptr()
        e.set_stream(st.cuda_stream)
        assert e.stream_ptr() == st.cuda_stream != own
        e.upload(pos, vel)
        pbfx.check(lib.pbf_ensemble_step(e.h, 5), "ensemble step")  # asynchronous, on st
        st.synchronize()
        e.set_stream(None)
        assert e.stream_ptr() == own
        e.step(3)
        got = e.download()
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(got[1], ref[1])
