"""The fused GB300 step (pbf_create / pbf_step) vs the CPU oracle step.

Per step, from the same state: sorted keys, permutation and cell tables
bit-exact; lambda of a single iteration bit-exact; positions, the last
iteration's lambda and velocities within the bars of tests/parity.py (the
oracle's powf is the C library's, CUDA's is not correctly rounded).
Multi-step runs compare each step from the GPU's own state.  Full-size runs
are checked through properties that do not depend on size.
"""
import ctypes as C

import numpy as np
import pytest

import pbfx
from parity import STEP_LAMBDA_FLOOR, STEP_POS, assert_velocities_close, step_lambda_tol

pytestmark = pytest.mark.gpu


def c1_scene(lib, iters=2):
    p = pbfx.dam_break_params((1.0, 1.0, 1.0), iters, 32 ** 3)
    pos = pbfx.seed_lattice(lib, 32, 32, 32, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    return p, pos, np.zeros_like(pos)


def compare_step(lib, orc, p, pos, vel, hashed, check_lambda=True):
    iters = p.solverIters
    with pbfx.Sim(lib, p, hashed=hashed) as s:
        s.upload(pos, vel)
        s.step()
        gpos, gvel = s.download()
        ks, perm = s.fetch(pbfx.DBG_KEYS_SORTED), s.fetch(pbfx.DBG_PERM)
        lam = s.fetch(pbfx.DBG_LAMBDA)
        if hashed:
            m = int(s.fetch(pbfx.DBG_COMPACT_COUNT)[0])
            uk = s.fetch(pbfx.DBG_UNIQUE_KEYS)[:m]
            off = s.fetch(pbfx.DBG_OFFSETS)[: m + 1]
        else:
            st, en = s.fetch(pbfx.DBG_CELL_START), s.fetch(pbfx.DBG_CELL_END)
    opos, ovel = pos.copy(), vel.copy()
    tr = pbfx.oracle_step(pbfx.load_oracle(), p, hashed, opos, ovel)
    np.testing.assert_array_equal(ks, tr["keys_sorted"])
    np.testing.assert_array_equal(perm, tr["perm"])
    if hashed:
        np.testing.assert_array_equal(uk, tr["unique_keys"])
        np.testing.assert_array_equal(off, tr["offsets"])
    else:
        np.testing.assert_array_equal(st, tr["cell_start"])
        np.testing.assert_array_equal(en, tr["cell_end"])
    if check_lambda:
        if iters == 1:
            np.testing.assert_array_equal(lam, tr["lambda"])  # from the prediction: exact
        else:
            pbfx.assert_close(lam, tr["lambda"], step_lambda_tol(iters), "lambda", floor_frac=STEP_LAMBDA_FLOOR)
    if iters == 0:
        np.testing.assert_array_equal(gpos, opos)
        np.testing.assert_array_equal(gvel, ovel)
    pbfx.assert_close(gpos, opos, STEP_POS, "positions")
    assert_velocities_close(gvel, ovel, opos, p.dt)
    assert np.all(gpos[:, 3] == 1.0) and np.all(gvel[:, 3] == 0.0)
    return gpos, gvel


@pytest.mark.parametrize("hashed", [True, False])
@pytest.mark.parametrize("iters", [0, 1, 2, 4])
def test_step_from_lattice(gpu, lib, orc, hashed, iters):
    p, pos, vel = c1_scene(lib, iters)
    compare_step(lib, orc, p, pos, vel, hashed, check_lambda=iters > 0)


@pytest.mark.parametrize("hashed", [True, False])
def test_step_by_step_over_a_run(gpu, lib, orc, hashed):
    """60 GPU steps; every 6th step is re-done by the oracle from the GPU state."""
    p, pos, vel = c1_scene(lib)
    with pbfx.Sim(lib, p, hashed=hashed) as s:
        s.upload(pos, vel)
        for k in range(60):
            if k % 6 == 0:
                cur_pos, cur_vel = s.download()
                compare_step(lib, orc, p, cur_pos, cur_vel, hashed)
            s.step()


# Boxes whose grids have 1,023, 1,024, 1,025 and 2,048 cells (the lower-bound
# table holds numCells + 1 entries and is filled in blocks of 1,024) and 125.
EDGE_BOXES = [(0.375, 0.03, 0.125), (0.1875, 0.0875, 0.0875), (0.5, 0.05, 0.05), (0.1875, 0.1875, 0.0875),
              (0.05, 0.05, 0.05)]


@pytest.mark.parametrize("box", EDGE_BOXES)
@pytest.mark.parametrize("corner", ["min", "max"])
def test_dense_cell_tables_at_block_edges(gpu, lib, orc, box, corner):
    """A few particles packed in the first cells (long empty tail) or in the
    last cells (long empty head) of grids sized around the fill's blocks."""
    p = pbfx.dam_break_params(box, 1, 18)
    assert pbfx.num_cells(p) in (1023, 1024, 1025, 2048, 125)
    dims = (3, 2, 3)
    if corner == "min":
        origin = (0.005, 0.005, 0.005)
    else:
        origin = tuple(b - 0.005 - (n - 1) * 0.01 for b, n in zip(box, dims))
    pos = pbfx.seed_lattice(lib, *dims, origin, 0.01, 0.0005, 0xC0FFEE, p)
    compare_step(lib, orc, p, pos, np.zeros_like(pos), hashed=False)


def test_xsph_disabled_and_restitution(gpu, lib, orc):
    p, pos, vel = c1_scene(lib)
    p.xsph_c = 0.0
    p.boundaryRestitution = 0.5
    rng = np.random.default_rng(2)
    vel[:, :3] = rng.normal(scale=2.0, size=(pos.shape[0], 3)).astype(np.float32)
    compare_step(lib, orc, p, pos, vel, True)


def test_neighbour_cap_engaged(gpu, lib, orc):
    """A compressed state with the cap at 8 neighbours."""
    p, pos, vel = c1_scene(lib)
    for _ in range(30):
        pbfx.oracle_step(orc, p, True, pos, vel, trace=False)
    p.maxNeighbors = 8
    compare_step(lib, orc, p, pos, vel, True)


def test_parameter_change_between_steps(gpu, lib, orc):
    """Dynamic (gravity, dt) and structural (solverIters) changes take effect."""
    p, pos, vel = c1_scene(lib)
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.upload(pos, vel)
        s.step()
        p2 = pbfx.dam_break_params((1.0, 1.0, 1.0), 3, 32 ** 3)
        p2.gravity.x = 2.0
        p2.dt = 1.0 / 240.0
        a_pos, a_vel = s.download()
        s.step(params=p2)
        gpos, gvel = s.download()
    opos, ovel = a_pos.copy(), a_vel.copy()
    pbfx.oracle_step(orc, p2, True, opos, ovel, trace=False)
    pbfx.assert_close(gpos, opos, STEP_POS, "positions")
    assert_velocities_close(gvel, ovel, opos, p2.dt)


def test_deterministic(gpu, lib):
    p, pos, vel = c1_scene(lib)
    outs = []
    for _ in range(2):
        with pbfx.Sim(lib, p, hashed=True) as s:
            s.upload(pos, vel)
            s.step(10)
            outs.append(s.download())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_density_stats_vs_fp64_oracle(gpu, lib, orc):
    p, pos, vel = c1_scene(lib)
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.upload(pos, vel)
        for k in range(3):
            st = s.density_stats()
            cur, _ = s.download()
            o = (C.c_double * 4)()
            orc.oracle_density_stats_f32pos(C.byref(p), pbfx.ptr(cur), cur.shape[0], C.byref(o))
            np.testing.assert_allclose(st[0], o[0], rtol=1e-5, atol=1e-6)
            np.testing.assert_allclose(st[1], o[1], rtol=1e-5, atol=1e-6)
            np.testing.assert_allclose(st[2], o[2], rtol=1e-5, atol=1e-6)
            assert st[3] == pytest.approx(o[3], rel=1e-4)  # r^2 == h^2 ties may differ FP32 vs FP64
            s.step(10)


def test_c2_full_size_properties(gpu, lib):
    """1,048,576 particles (128x64x128 lattice, [0,2]x[0,1]x[0,2]): sortedness,
    permutation, table consistency and finite state after 20 steps."""
    n = 128 * 64 * 128
    p = pbfx.dam_break_params((2.0, 1.0, 2.0), 2, n)
    pos = pbfx.seed_lattice(lib, 128, 64, 128, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.upload(pos, np.zeros_like(pos))
        s.step(20)
        ks, perm = s.fetch(pbfx.DBG_KEYS_SORTED), s.fetch(pbfx.DBG_PERM)
        m = int(s.fetch(pbfx.DBG_COMPACT_COUNT)[0])
        uk, off = s.fetch(pbfx.DBG_UNIQUE_KEYS)[:m], s.fetch(pbfx.DBG_OFFSETS)[: m + 1]
        st, en = s.fetch(pbfx.DBG_CELL_START), s.fetch(pbfx.DBG_CELL_END)
        gpos, gvel = s.download()
    assert np.all(np.diff(ks.astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(perm), np.arange(n, dtype=np.uint32))
    # stable: equal keys keep ascending particle ids
    same = ks[1:] == ks[:-1]
    assert np.all(perm[1:][same] > perm[:-1][same])
    u, first = np.unique(ks, return_index=True)
    assert m == len(u) and np.array_equal(uk, u) and np.array_equal(off[:-1], first) and off[-1] == n
    occ = st != 0xFFFFFFFF
    assert occ.sum() == m and np.array_equal(st[occ], first) and np.array_equal(en[occ], np.append(first[1:], n))
    assert np.all(np.isfinite(gpos)) and np.all(np.isfinite(gvel))
    assert gpos[:, :3].min() >= 0.0 and gpos[:, 0].max() <= 2.0 and gpos[:, 1].max() <= 1.0


def test_step_host_matches_device_path(gpu, lib):
    p, pos, vel = c1_scene(lib)
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.upload(pos, vel)
        s.step(1)
        a = s.download()
    hp, hv = pos.copy(), vel.copy()
    with pbfx.Sim(lib, p, hashed=True) as s:
        pbfx.check(lib.pbf_step_host(s.h, None, pbfx.ptr(hp), pbfx.ptr(hv)))
    assert np.array_equal(a[0], hp) and np.array_equal(a[1], hv)


@pytest.mark.parametrize("hashed", [True, False])
def test_nonfinite_state_is_reported(gpu, lib, hashed):
    """A NaN in the state is reported as PBF_ERR_NONFINITE by pbf_synchronize
    (cell keys clamp it into the grid; nothing faults), the flag clears once
    reported, and a clean state steps without error again."""
    p, pos, vel = c1_scene(lib)
    bad = pos.copy()
    bad[1234, 1] = np.nan
    with pbfx.Sim(lib, p, hashed=hashed) as s:
        s.upload(bad, vel)
        assert lib.pbf_step_n(s.h, None, 1) == pbfx.PBF_OK
        assert lib.pbf_synchronize(s.h) == pbfx.PBF_ERR_NONFINITE
        assert lib.pbf_synchronize(s.h) == pbfx.PBF_OK
        s.upload(pos, vel)
        assert lib.pbf_step_n(s.h, None, 2) == pbfx.PBF_OK
        assert lib.pbf_synchronize(s.h) == pbfx.PBF_OK


def test_caller_stream(gpu, lib):
    """pbf_set_stream: steps enqueued on a caller's stream give the same state;
    NULL returns to the handle's own stream."""
    torch = pytest.importorskip("torch")
    p, pos, vel = c1_scene(lib)
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.upload(pos, vel)
        s.step(6)
        ref = s.download()
    st = torch.cuda.Stream()
    with pbfx.Sim(lib, p, hashed=True) as s:
        own = s.stream_ptr()
        s.set_stream(st.cuda_stream)
        assert s.stream_ptr() == st.cuda_stream != own
        s.upload(pos, vel)
        for _ in range(5):
            pbfx.check(lib.pbf_step(s.h, None), "step")  # asynchronous, on st
        done = torch.cuda.Event()
        done.record(st)
        done.synchronize()
        assert st.query()
        s.set_stream(None)
        assert s.stream_ptr() == own
        s.step(1)
        got = s.download()
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(got[1], ref[1])
