"""PBF_MATH_FAST: the delta pass's s_corr power for n = 4 from error-free
products (ratio^4 correctly rounded except next to a tie) instead of CUDA's
powf.

Per step, from the same state, against the FP32 oracle: sorted keys,
permutation and cell tables bit-exact (they come from the prediction, before
any neighbour arithmetic), the first iteration's lambda bit-exact (the lambda
pass is the exact mode's); the last iteration's lambda, positions and
velocities within the bars of tests/parity.py (spec: 1e-5 relative on
state).  The power itself is checked against a correctly rounded x^4.
"""
import numpy as np
import pytest

import pbfx
from parity import STEP_LAMBDA_FLOOR, STEP_POS, assert_velocities_close, step_lambda_tol

pytestmark = pytest.mark.gpu


def c1_scene(lib, iters=2):
    p = pbfx.dam_break_params((1.0, 1.0, 1.0), iters, 32 ** 3)
    pos = pbfx.seed_lattice(lib, 32, 32, 32, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    return p, pos, np.zeros_like(pos)


def fast_step_vs_oracle(s, orc, p, hashed):
    """One fast-mode step of Sim s from its current state, checked against
    the oracle stepped from the same state."""
    cur_pos, cur_vel = s.download()
    opos, ovel = cur_pos.copy(), cur_vel.copy()
    tr = pbfx.oracle_step(orc, p, hashed, opos, ovel)
    s.step()
    np.testing.assert_array_equal(s.fetch(pbfx.DBG_KEYS_SORTED), tr["keys_sorted"])
    np.testing.assert_array_equal(s.fetch(pbfx.DBG_PERM), tr["perm"])
    if hashed:
        m = int(s.fetch(pbfx.DBG_COMPACT_COUNT)[0])
        np.testing.assert_array_equal(s.fetch(pbfx.DBG_UNIQUE_KEYS)[:m], tr["unique_keys"])
        np.testing.assert_array_equal(s.fetch(pbfx.DBG_OFFSETS)[: m + 1], tr["offsets"])
    else:
        np.testing.assert_array_equal(s.fetch(pbfx.DBG_CELL_START), tr["cell_start"])
        np.testing.assert_array_equal(s.fetch(pbfx.DBG_CELL_END), tr["cell_end"])
    gpos, gvel = s.download()
    if p.solverIters == 1:
        np.testing.assert_array_equal(s.fetch(pbfx.DBG_LAMBDA), tr["lambda"])  # from the prediction: exact
    elif p.solverIters > 1:
        pbfx.assert_close(s.fetch(pbfx.DBG_LAMBDA), tr["lambda"], step_lambda_tol(p.solverIters), "lambda",
                          floor_frac=STEP_LAMBDA_FLOOR)
    pbfx.assert_close(gpos, opos, STEP_POS, "positions")
    assert_velocities_close(gvel, ovel, opos, p.dt)
    assert np.all(gpos[:, 3] == 1.0) and np.all(gvel[:, 3] == 0.0)


@pytest.mark.parametrize("hashed", [True, False])
@pytest.mark.parametrize("iters", [1, 2, 4])
def test_fast_step_from_lattice(gpu, lib, orc, hashed, iters):
    p, pos, vel = c1_scene(lib, iters)
    with pbfx.Sim(lib, p, hashed=hashed) as s:
        s.set_math_mode(pbfx.PBF_MATH_FAST)
        assert s.math_mode() == pbfx.PBF_MATH_FAST
        s.upload(pos, vel)
        fast_step_vs_oracle(s, orc, p, hashed)


@pytest.mark.parametrize("hashed", [True, False])
def test_fast_step_by_step_over_a_run(gpu, lib, orc, hashed):
    """60 fast steps; every 6th is checked against the oracle from the GPU state."""
    p, pos, vel = c1_scene(lib)
    with pbfx.Sim(lib, p, hashed=hashed) as s:
        s.set_math_mode(pbfx.PBF_MATH_FAST)
        s.upload(pos, vel)
        for k in range(60):
            if k % 6 == 0:
                fast_step_vs_oracle(s, orc, p, hashed)
            else:
                s.step()


def test_fast_cap_and_restitution(gpu, lib, orc):
    """A compressed state with the neighbour cap at 8, restitution 0.5 and
    random velocities."""
    p, pos, vel = c1_scene(lib)
    for _ in range(30):
        pbfx.oracle_step(orc, p, True, pos, vel, trace=False)
    p.maxNeighbors = 8
    p.boundaryRestitution = 0.5
    rng = np.random.default_rng(5)
    vel[:, :3] += rng.normal(scale=0.5, size=(pos.shape[0], 3)).astype(np.float32)
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.set_math_mode(pbfx.PBF_MATH_FAST)
        s.upload(pos, vel)
        fast_step_vs_oracle(s, orc, p, True)


@pytest.mark.parametrize("scorr_n", [4.0, 3.0])
def test_fast_scorr_exponents(gpu, lib, orc, scorr_n):
    """n = 4 takes the product form, other exponents powf."""
    p, pos, vel = c1_scene(lib)
    p.pbf.scorr_n = scorr_n
    for _ in range(10):
        pbfx.oracle_step(orc, p, True, pos, vel, trace=False)
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.set_math_mode(pbfx.PBF_MATH_FAST)
        s.upload(pos, vel)
        fast_step_vs_oracle(s, orc, p, True)


def test_fast_c2_in_the_timed_window(gpu, lib, orc):
    """The bench workload (1,048,576 particles, 2 iterations, hashed): steps 6,
    15 and 24 of a fast-mode run, each against the oracle from the GPU state."""
    n = 128 * 64 * 128
    p = pbfx.dam_break_params((2.0, 1.0, 2.0), 2, n)
    pos = pbfx.seed_lattice(lib, 128, 64, 128, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.set_math_mode(pbfx.PBF_MATH_FAST)
        s.upload(pos, np.zeros_like(pos))
        for k in range(25):
            if k in (5, 14, 23):
                fast_step_vs_oracle(s, orc, p, True)
            else:
                s.step()


def test_fast_and_exact_modes_switch(gpu, lib):
    """Switching modes re-captures the step: a fast step differs from the
    exact one in the last bits, and exact steps after fast ones are the exact
    path's (bit-identical to a run that never switched)."""
    p, pos, vel = c1_scene(lib)
    with pbfx.Sim(lib, p, hashed=True) as a, pbfx.Sim(lib, p, hashed=True) as b:
        a.upload(pos, vel)
        b.upload(pos, vel)
        b.set_math_mode(pbfx.PBF_MATH_FAST)
        b.step(1)
        fast_pos, _ = b.download()
        a.step(1)
        exact_pos, exact_vel = a.download()
        assert not np.array_equal(fast_pos, exact_pos)  # different arithmetic
        pbfx.assert_close(fast_pos, exact_pos, STEP_POS, "fast vs exact after a step")
        b.upload(exact_pos, exact_vel)
        b.set_math_mode(pbfx.PBF_MATH_EXACT)
        a.step(2)
        b.step(2)
        pa, va = a.download()
        pb, vb = b.download()
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)


def test_fast_ensemble_against_oracle(gpu, lib, orc):
    """Three seeded ensemble scenes (tilted gravity, 3 iterations) in fast mode,
    every scene checked per step against the oracle."""
    scenes, pos = pbfx.ensemble_scenes(lib, 3, seed=0xFA57, iters_choices=(3,))
    with pbfx.Ensemble(lib, scenes) as e:
        e.set_math_mode(pbfx.PBF_MATH_FAST)
        e.upload(pos, np.zeros_like(pos))
        off = e.offsets.astype(np.int64)
        for k in range(9):
            cur_pos, cur_vel = e.download()
            e.step()
            if k % 4:
                continue
            gpos, gvel = e.download()
            for si, sc in enumerate(scenes):
                a, b = off[si], off[si + 1]
                opos, ovel = cur_pos[a:b].copy(), cur_vel[a:b].copy()
                pbfx.oracle_step(orc, sc, True, opos, ovel, trace=False)
                pbfx.assert_close(gpos[a:b], opos, STEP_POS, "scene %d positions" % si)
                assert_velocities_close(gvel[a:b], ovel, opos, sc.dt)


def test_compensated_pow4_is_correctly_rounded(gpu, lib):
    """The fast mode's x^4 against x^4 rounded once from an exact value, on
    2^22 random floats in [0, 2] plus powers of two and their neighbours:
    equal wherever x^4 is not within 2^-20 ulp of a rounding tie."""
    import ctypes as C

    torch = gpu
    rng = np.random.default_rng(4)
    x = np.concatenate([rng.uniform(0.0, 2.0, 1 << 22).astype(np.float32),
                        np.ldexp(np.float32(1.0), np.arange(-30, 30)).astype(np.float32),
                        np.nextafter(np.ldexp(np.float32(1.0), np.arange(-30, 30)).astype(np.float32),
                                     np.float32(np.inf)),
                        np.float32([0.0, 1.0, 0.5, 0.25])])
    a = torch.from_numpy(x).cuda()
    out = torch.empty_like(a)
    pbfx.check(lib.pbf_debug_eval_math(3, C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()),
                                       C.c_void_p(out.data_ptr()), x.size), "eval_math")
    got = out.cpu().numpy()
    # x^2 is exact in float64 (48 significant bits); x^4 = (x^2)^2 rounded to
    # float64 is within 2^-53 relative, so rounding it to float32 gives the
    # correctly rounded x^4 unless x^4 lies that close to a float32 tie.
    x64 = x.astype(np.float64)
    q = x64 * x64
    want64 = q * q
    want = want64.astype(np.float32)
    ulp = np.spacing(want).astype(np.float64)
    frac = np.abs(want64 - want.astype(np.float64)) / np.where(ulp > 0, ulp, 1.0)
    near_tie = np.abs(frac - 0.5) < 2.0 ** -20
    bad = (got != want) & ~near_tie
    assert not bad.any(), "x = %r: got %r, want %r" % (x[bad][:5], got[bad][:5], want[bad][:5])
