"""The batched adjoint (pbf_forward_batch / pbf_backward_batch) against the
same scenes differentiated one at a time (pbf_forward / pbf_backward).

A batch enqueues step n of every scene before step n + 1 of any, each scene
on its own stream, and synchronises once; the kernels and their order within
a scene are those of the single-scene calls.  Three scenes of different sizes
and iteration counts (XSPH on, s_corr on, the reference's default constants),
6 steps with checkpoints every 3: the final states, dL/d(initial positions),
dL/d(initial velocities) and dL/d(xsph_c) are the same bits both ways.
"""
import ctypes as C

import numpy as np
import pytest

import pbfx

pytestmark = pytest.mark.gpu

SCENES = [((12, 12, 12), 2, 0xA1), ((10, 14, 10), 3, 0xA2), ((16, 8, 12), 1, 0xA3)]
STEPS, EVERY = 6, 3


def scene(lib, dims, iters, seed):
    nx, ny, nz = dims
    p = pbfx.dam_break_params((0.5, 0.5, 0.5), iters, nx * ny * nz)
    pos = pbfx.seed_lattice(lib, nx, ny, nz, (0.005, 0.005, 0.005), 0.01, 0.0005, seed, p)
    rng = np.random.default_rng(seed)
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.uniform(-0.2, 0.2, (pos.shape[0], 3))
    pbar = np.zeros_like(pos)
    vbar = np.zeros_like(pos)
    pbar[:, :3] = rng.standard_normal((pos.shape[0], 3))
    vbar[:, :3] = rng.standard_normal((pos.shape[0], 3))
    return p, pos, vel, pbar, vbar


def test_batch_matches_scene_by_scene(gpu, lib):
    torch = gpu
    data = [scene(lib, *sc) for sc in SCENES]

    def run(batched):
        sims = [pbfx.Sim(lib, p, hashed=True) for p, *_ in data]
        try:
            for s, (p, pos, vel, _, _) in zip(sims, data):
                s.upload(pos, vel)
            pb = [torch.from_numpy(d[3]).cuda() for d in data]
            vb = [torch.from_numpy(d[4]).cuda() for d in data]
            gp = [torch.zeros_like(x) for x in pb]
            gv = [torch.zeros_like(x) for x in pb]
            if batched:
                tapes = pbfx.forward_batch(lib, sims, STEPS, EVERY)
            else:
                tapes = []
                for s in sims:
                    t = C.c_void_p()
                    pbfx.check(lib.pbf_forward(s.h, STEPS, EVERY, C.byref(t)), "forward")
                    tapes.append(t)
            try:
                finals = [s.download() for s in sims]
                if batched:
                    cb = pbfx.backward_batch(lib, tapes, [x.data_ptr() for x in pb], [x.data_ptr() for x in vb],
                                             [x.data_ptr() for x in gp], [x.data_ptr() for x in gv])
                else:
                    cb = []
                    for t, a, b, c, d in zip(tapes, pb, vb, gp, gv):
                        g = C.c_float()
                        pbfx.check(lib.pbf_backward(t, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                                    C.c_void_p(c.data_ptr()), C.c_void_p(d.data_ptr()),
                                                    C.byref(g)), "backward")
                        cb.append(g.value)
                torch.cuda.synchronize()
                return finals, [x.cpu().numpy() for x in gp], [x.cpu().numpy() for x in gv], cb
            finally:
                for t in tapes:
                    lib.pbf_tape_destroy(t)
        finally:
            for s in sims:
                s.close()

    one = run(False)
    many = run(True)
    for k in range(len(SCENES)):
        np.testing.assert_array_equal(many[0][k][0], one[0][k][0])
        np.testing.assert_array_equal(many[0][k][1], one[0][k][1])
        np.testing.assert_array_equal(many[1][k], one[1][k])
        np.testing.assert_array_equal(many[2][k], one[2][k])
        assert many[3][k] == one[3][k]
        assert np.abs(one[1][k][:, :3]).max() > 0 and np.isfinite(one[1][k]).all()


def test_batch_rejects_bad_arguments(gpu, lib):
    p, pos, vel, _, _ = scene(lib, (8, 8, 8), 2, 0xB1)
    k2 = (C.c_void_p * 2)()
    assert lib.pbf_forward_batch(None, 1, 2, 1, k2) == pbfx.PBF_ERR_INVALID
    with pbfx.Sim(lib, p) as a, pbfx.Sim(lib, p) as b:
        a.upload(pos, vel)
        b.upload(pos, vel)
        dup = (C.c_void_p * 2)(a.h.value, a.h.value)
        k2[0] = k2[1] = 1  # overwritten with NULL on failure
        assert lib.pbf_forward_batch(dup, 2, 2, 1, k2) == pbfx.PBF_ERR_INVALID
        assert k2[0] is None and k2[1] is None
        assert lib.pbf_forward_batch(dup, 0, 2, 1, k2) == pbfx.PBF_ERR_INVALID
        both = (C.c_void_p * 2)(a.h.value, b.h.value)
        assert lib.pbf_forward_batch(both, 2, 0, 1, k2) == pbfx.PBF_ERR_INVALID
        ta, tb = C.c_void_p(), C.c_void_p()
        pbfx.check(lib.pbf_forward(a.h, 2, 1, C.byref(ta)), "forward")
        pbfx.check(lib.pbf_forward(b.h, 3, 1, C.byref(tb)), "forward")
        try:
            bar = gpu.zeros((pos.shape[0], 4), dtype=gpu.float32, device="cuda")
            ptrs = (C.c_void_p * 2)(bar.data_ptr(), bar.data_ptr())
            mixed = (C.c_void_p * 2)(ta.value, tb.value)
            # different step counts in one batch
            assert lib.pbf_backward_batch(mixed, 2, ptrs, ptrs, None, None, None) == pbfx.PBF_ERR_INVALID
            same = (C.c_void_p * 2)(ta.value, ta.value)
            assert lib.pbf_backward_batch(same, 2, ptrs, ptrs, None, None, None) == pbfx.PBF_ERR_INVALID
            assert lib.pbf_backward_batch(mixed, 1, None, ptrs, None, None, None) == pbfx.PBF_ERR_INVALID
            # one tape alone through the batch entry, without outputs
            one = (C.c_void_p * 1)(ta.value)
            assert lib.pbf_backward_batch(one, 1, ptrs, ptrs, None, None, None) == pbfx.PBF_OK
        finally:
            lib.pbf_tape_destroy(ta)
            lib.pbf_tape_destroy(tb)
