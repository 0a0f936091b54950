"""Parity with the reference itself.

tests/golden/ref_*.npz hold one step of the reference's own CUDA kernels
(compiled from its sources, driven in its phase order by
oracle/ref/ref_harness.cu; written by oracle/ref/make_ref_fixtures.py).

* CPU: the oracle reproduces them - sorted keys, permutation and cell tables
  bit-exact, positions / lambda / velocities within the bars of
  tests/parity.py.  This pins the oracle to the reference.
* GPU: the fused GB300 step reproduces them bit for bit.
* GPU, when the reference's device images are present: 40-step trajectories
  of the fused step and of the reference kernels at C1 size stay
  bit-identical.
"""
import glob
import os

import numpy as np
import pytest

import pbfx
from parity import STEP_LAMBDA_FLOOR, STEP_POS, assert_velocities_close, step_lambda_tol

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "ref_*.npz")))


def load_fixture(path):
    z = np.load(path)
    p = pbfx.SimParams.from_buffer_copy(z["params"].tobytes())
    return p, bool(int(z["hashed"])), z


def check_against(z, hashed, out_pos, out_vel, tr, exact, dt):
    np.testing.assert_array_equal(tr["keys_sorted"], z["keys_sorted"])
    np.testing.assert_array_equal(tr["perm"], z["perm"])
    if hashed:
        np.testing.assert_array_equal(tr["unique_keys"], z["unique_keys"])
        np.testing.assert_array_equal(tr["offsets"], z["offsets"])
    else:
        np.testing.assert_array_equal(tr["cell_start"], z["cell_start"])
        np.testing.assert_array_equal(tr["cell_end"], z["cell_end"])
    if exact:
        np.testing.assert_array_equal(tr["lambda"], z["lambda"])
        np.testing.assert_array_equal(out_pos, z["pos_out"])
        np.testing.assert_array_equal(out_vel, z["vel_out"])
    else:
        pbfx.assert_close(out_pos, z["pos_out"], STEP_POS, "positions")
        pbfx.assert_close(tr["lambda"], z["lambda"], step_lambda_tol(2), "lambda", floor_frac=STEP_LAMBDA_FLOOR)
        assert_velocities_close(out_vel, z["vel_out"], z["pos_out"], dt)


def test_fixtures_present():
    assert len(FIXTURES) >= 6, "reference fixtures missing: run oracle/ref/make_ref_fixtures.py on a GPU"


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[4:-4] for f in FIXTURES])
def test_oracle_reproduces_reference(orc, path):
    p, hashed, z = load_fixture(path)
    pos, vel = z["pos_in"].copy(), z["vel_in"].copy()
    tr = pbfx.oracle_step(orc, p, hashed, pos, vel)
    check_against(z, hashed, pos, vel, tr, exact=False, dt=p.dt)


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[4:-4] for f in FIXTURES])
def test_fused_step_reproduces_reference(gpu, lib, path):
    p, hashed, z = load_fixture(path)
    with pbfx.Sim(lib, p, hashed=hashed) as s:
        s.upload(z["pos_in"], z["vel_in"])
        s.step()
        pos, vel = s.download()
        tr = {"keys_sorted": s.fetch(pbfx.DBG_KEYS_SORTED), "perm": s.fetch(pbfx.DBG_PERM),
              "lambda": s.fetch(pbfx.DBG_LAMBDA)}
        if hashed:
            m = int(s.fetch(pbfx.DBG_COMPACT_COUNT)[0])
            tr["unique_keys"] = s.fetch(pbfx.DBG_UNIQUE_KEYS)[:m]
            tr["offsets"] = s.fetch(pbfx.DBG_OFFSETS)[: m + 1]
        else:
            tr["cell_start"] = s.fetch(pbfx.DBG_CELL_START)
            tr["cell_end"] = s.fetch(pbfx.DBG_CELL_END)
    check_against(z, hashed, pos, vel, tr, exact=True, dt=p.dt)


@pytest.mark.gpu
@pytest.mark.parametrize("hashed", [True, False])
def test_live_reference_kernels_c1(gpu, lib, hashed):
    """The same 40-step C1 run through the reference kernels and through the
    fused GB300 step: states, sorted keys, permutation and lambda identical
    at every 8th step, and the final states identical."""
    ref = pbfx.load_ref()
    if ref is None:
        pytest.skip("reference device images not present in this checkout")
    p = pbfx.dam_break_params((1.0, 1.0, 1.0), 2, 32 ** 3)
    pos = pbfx.seed_lattice(lib, 32, 32, 32, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    rp, rv = pos.copy(), np.zeros_like(pos)
    with pbfx.Sim(lib, p, hashed=hashed) as s:
        s.upload(pos, np.zeros_like(pos))
        for k in range(40):
            rtr = pbfx.ref_step(ref, p, hashed, rp, rv, trace=(k % 8 == 0))
            s.step()
            if k % 8 == 0:
                gp, gv = s.download()
                np.testing.assert_array_equal(s.fetch(pbfx.DBG_KEYS_SORTED), rtr["keys_sorted"])
                np.testing.assert_array_equal(s.fetch(pbfx.DBG_PERM), rtr["perm"])
                np.testing.assert_array_equal(s.fetch(pbfx.DBG_LAMBDA), rtr["lambda"])
                np.testing.assert_array_equal(gp, rp)
                np.testing.assert_array_equal(gv, rv)
        gp, gv = s.download()
    np.testing.assert_array_equal(gp, rp)
    np.testing.assert_array_equal(gv, rv)
