"""Tile shapes of the neighbour passes and their autotuner.

A tile shape sets how many consecutive sorted particles a CTA of the list
passes takes and how many neighbour slots it may stage in shared memory.
Only which tiles are staged (and so where neighbour data is read from)
depends on it, so every shape must give the same state bit for bit.  The
autotuner times each shape from the current state and must leave that state
as it found it.
"""
import numpy as np
import pytest

import pbfx
from test_gpu_ensemble import mixed_scenes

pytestmark = pytest.mark.gpu


def scene(lib, iters=2, dims=(30, 31, 33)):
    n = dims[0] * dims[1] * dims[2]
    p = pbfx.dam_break_params((1.0, 1.0, 1.0), iters, n)
    pos = pbfx.seed_lattice(lib, *dims, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    return p, pos, np.zeros_like(pos)


def run(lib, p, pos, vel, hashed, shape, steps, cap=None):
    with pbfx.Sim(lib, p, hashed=hashed) as s:
        if cap is not None:
            s.set_list_capacity(cap)
        s.set_tile_shape(shape)
        assert s.tile_shape() == shape
        s.upload(pos, vel)
        s.step(steps)
        gp, gv = s.download()
        return gp, gv, s.fetch(pbfx.DBG_LAMBDA)


def kept_or_fastest(ms, chosen, before):
    """The tuner keeps the current shape unless another is at least 2% faster."""
    best = min(range(len(ms)), key=lambda i: ms[i])
    if ms[best] < ms[before] * 0.98:
        return chosen == best
    return chosen == before


def assert_same(a, b):
    for x, y, what in zip(a, b, ("positions", "velocities", "lambda")):
        np.testing.assert_array_equal(x, y, err_msg=what)


def test_shapes_are_listed(lib):
    shapes = pbfx.tile_shapes(lib)
    assert shapes[0] == (128, 1536)
    assert len(shapes) == len(set(shapes)) >= 2
    assert all(t % 32 == 0 and st >= t for t, st in shapes)


@pytest.mark.parametrize("hashed", [True, False])
@pytest.mark.parametrize("iters", [2, 3])
def test_every_tile_shape_gives_the_same_state(gpu, lib, hashed, iters):
    p, pos, vel = scene(lib, iters)
    ref = run(lib, p, pos, vel, hashed, 0, 30)
    for shape in range(1, len(pbfx.tile_shapes(lib))):
        assert_same(run(lib, p, pos, vel, hashed, shape, 30), ref)


def test_tile_shapes_with_overflowing_lists(gpu, lib):
    """Capacity 64: some warps walk lists, the others the stencil."""
    p, pos, vel = scene(lib)
    ref = run(lib, p, pos, vel, True, 0, 20, cap=0)
    for shape in range(len(pbfx.tile_shapes(lib))):
        assert_same(run(lib, p, pos, vel, True, shape, 20, cap=64), ref)


def test_unknown_shape_is_refused(gpu, lib):
    p, pos, vel = scene(lib)
    with pbfx.Sim(lib, p) as s:
        for bad in (-1, len(pbfx.tile_shapes(lib))):
            with pytest.raises(RuntimeError):
                s.set_tile_shape(bad)
        assert s.tile_shape() == 0


def test_autotune_restores_the_state(gpu, lib):
    p, pos, vel = scene(lib)
    with pbfx.Sim(lib, p) as s:
        s.upload(pos, vel)
        s.step(5)
        before = s.download()
        chosen, ms = s.autotune(steps=2)
        after = s.download()
        assert_same(after, before[:2])
        assert s.tile_shape() == chosen
        assert len(ms) == len(pbfx.tile_shapes(lib)) and all(m > 0 for m in ms)
        assert kept_or_fastest(ms, chosen, 0)
        s.step(5)
        tuned = s.download()
    untuned = run(lib, p, pos, vel, True, 0, 10)
    assert_same(tuned, untuned[:2])


def test_ensemble_shapes_and_autotune(gpu, lib):
    scenes, pos = mixed_scenes(lib)
    vel = np.zeros_like(pos)
    out = []
    for shape in range(len(pbfx.tile_shapes(lib))):
        with pbfx.Ensemble(lib, scenes) as e:
            e.set_tile_shape(shape)
            assert e.tile_shape() == shape
            e.upload(pos, vel)
            e.step(20)
            out.append(e.download())
    for o in out[1:]:
        assert_same(o, out[0])
    with pbfx.Ensemble(lib, scenes) as e:
        e.upload(pos, vel)
        e.step(10)
        before = e.download()
        chosen, ms = e.autotune(steps=2)
        assert_same(e.download(), before)
        assert e.tile_shape() == chosen and kept_or_fastest(ms, chosen, 0)
        e.step(10)
        assert_same(e.download(), out[0])
        with pytest.raises(RuntimeError):
            e.set_tile_shape(len(ms))
