"""Neighbour lists of the fused step vs the stencil walk they replace.

With the displacement clamp on, each solver pass walks a per-particle list
of the stencil candidates that were within the list radius when it was
built, instead of the 27-cell stencil.  The list holds every candidate the
pass can accept, in the stencil's order, so the state must be bit-identical
to the stencil walk (list capacity 0) after any number of steps, whatever
the capacity (overflowed lists make their warp walk the stencil), the number
of iterations a list spans, the grid mode and a particle count that leaves
partial warps.
"""
import numpy as np
import pytest

import pbfx

pytestmark = pytest.mark.gpu


def scene(lib, iters=2, dims=(30, 31, 33), clamp=None):
    n = dims[0] * dims[1] * dims[2]
    p = pbfx.dam_break_params((1.0, 1.0, 1.0), iters, n)
    if clamp is not None:
        p.pbf.disp_clamp_max_h = clamp
    pos = pbfx.seed_lattice(lib, *dims, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    return p, pos, np.zeros_like(pos)


def run(lib, p, pos, vel, hashed, cap, steps):
    """(pos, vel, lambda, list stats, launches per step) after `steps` steps."""
    with pbfx.Sim(lib, p, hashed=hashed) as s:
        if cap is not None:
            s.set_list_capacity(cap)
        s.upload(pos, vel)
        s.step(steps)
        gp, gv = s.download()
        lam = s.fetch(pbfx.DBG_LAMBDA)
        return gp, gv, lam, s.list_stats(), s.launches_per_step()


def assert_same(a, b):
    for x, y, what in zip(a[:3], b[:3], ("positions", "velocities", "lambda")):
        np.testing.assert_array_equal(x, y, err_msg=what)


@pytest.mark.parametrize("hashed", [True, False])
@pytest.mark.parametrize("iters", [1, 2, 3, 4])
def test_lists_match_the_stencil_walk(gpu, lib, hashed, iters):
    p, pos, vel = scene(lib, iters)
    walk = run(lib, p, pos, vel, hashed, 0, 40)
    lists = run(lib, p, pos, vel, hashed, None, 40)
    assert_same(lists, walk)
    cap, longest, overflowed = lists[3]
    assert cap == 512 and 0 < longest <= cap and overflowed == 0
    assert walk[3] == (0, 0, 0)
    # one list for the whole step: h + 2 * iters * 0.05 h <= 1.5 h
    assert lists[4] - walk[4] == 1


@pytest.mark.parametrize("which", ["all", "some"])
def test_overflowing_lists_fall_back_to_the_stencil(gpu, lib, which):
    """Capacity 8 (every list overflows) or half the longest list (some
    warps walk lists, others the stencil)."""
    p, pos, vel = scene(lib)
    walk = run(lib, p, pos, vel, True, 0, 30)
    cap = 8
    if which == "some":
        cap = max(8, (run(lib, p, pos, vel, True, None, 30)[3][1] // 2) & ~7)
    lists = run(lib, p, pos, vel, True, cap, 30)
    assert_same(lists, walk)
    c, longest, overflowed = lists[3]
    assert c == cap and longest > cap and overflowed > 0


@pytest.mark.parametrize("cap", [24, 32, 40])
def test_capacities_around_the_unbounded_emit(gpu, lib, cap):
    """From a capacity of 32, staged tiles write their 16-bit lists without a
    bound per lane (the list's 2 x capacity of room absorbs an emit that
    starts within the capacity); below it, every emit is bounded.  Lists
    overflow at these capacities, so the state must still equal the stencil
    walk's, and the counts of the other lists must not be disturbed."""
    p, pos, vel = scene(lib)
    walk = run(lib, p, pos, vel, True, 0, 30)
    lists = run(lib, p, pos, vel, True, cap, 30)
    assert_same(lists, walk)
    c, longest, overflowed = lists[3]
    assert c == cap and longest > cap and overflowed > 0


@pytest.mark.parametrize("iters, clamp, builds", [(3, 0.0, 1), (3, 0.02, 1), (6, 0.05, 2), (7, 0.05, 3),
                                                  (3, 0.1, 2), (4, 0.12, 2)])
def test_list_schedule_follows_the_displacement_clamp(gpu, lib, iters, clamp, builds):
    """One list for the step while h + 2 * iters * clamp * h <= 1.5 h;
    otherwise one per span of iterations (radius <= 1.25 h) and the commit
    walks the stencil: a list built after the first update may start outside
    the box, and the final boundary projection can move such a particle
    further than the remaining updates."""
    p, pos, vel = scene(lib, iters=iters, clamp=clamp)
    walk = run(lib, p, pos, vel, True, 0, 30)
    lists = run(lib, p, pos, vel, True, None, 30)
    assert_same(lists, walk)
    assert lists[3][1] > 0 and lists[3][2] == 0
    assert lists[4] - walk[4] == builds


@pytest.mark.parametrize("clamp_on, clamp", [(0, 0.05), (1, 0.3)])
def test_no_lists_without_a_displacement_bound(gpu, lib, clamp_on, clamp):
    """Clamp off (particles may move any distance), or 0.3 h per update with
    two iterations (one list would reach 2.2 h and a span would hold a single
    iteration): no list is built and every pass walks the stencil."""
    p, pos, vel = scene(lib, clamp=clamp)
    p.pbf.enable_disp_clamp = clamp_on
    walk = run(lib, p, pos, vel, True, 0, 20)
    lists = run(lib, p, pos, vel, True, None, 20)
    assert_same(lists, walk)
    assert lists[3][1] == 0 and lists[4] == walk[4]


def test_clamp_switched_off_between_steps(gpu, lib):
    """The graph is re-captured without list builds when the clamp goes off."""
    p, pos, vel = scene(lib)
    q = pbfx.dam_break_params((1.0, 1.0, 1.0), 2, pos.shape[0])
    q.pbf.enable_disp_clamp = 0
    out = []
    for cap in (0, None):
        with pbfx.Sim(lib, p, hashed=True) as s:
            if cap is not None:
                s.set_list_capacity(cap)
            s.upload(pos, vel)
            s.step(10)
            s.step(10, q)
            s.step(10, p)
            out.append(s.download())
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
