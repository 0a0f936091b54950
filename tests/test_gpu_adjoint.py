"""Adjoint of the step (pbf_forward / pbf_backward) vs FP64 finite differences.

Loss: mean squared difference between the SPH density on a grid of cell
centres after a few steps and a target density (the same measurement of a
run from seeded initial velocities).  Gradients w.r.t. initial velocities
and xsph_c from the GPU adjoint are compared with central differences of the
FP64 CPU oracle's step on the same scene, with the loss evaluated in FP64.

The reference's dynamics are numerically chaotic at its default constants:
its position correction carries no particle mass, so s_corr drives it ~100x
past the 0.05 h displacement clamp, and every particle moves 0.05 h per
iteration along a sum of large cancelling terms.  FP32 and FP64 trajectories
of the same scene separate ~10x per step (3e-7, 3e-6, 3e-5 m after 1, 2, 3
steps).  A gradient of the FP32 step can therefore match FP64 differences
only over a short horizon: the default constants are checked over 2 steps
(clamped displacements, s_corr), and a smooth regime (s_corr off, large
lambda epsilon: unclamped displacements, FP32/FP64 apart by 1e-6 m after 4
steps) over 4.  The block starts 5 cm from the walls so no clamp engages.
"""
import ctypes as C

import numpy as np
import pytest

import pbfx

RES = 16
# max |g - g_fd| / max |g_fd| over the checked coordinates.  The default
# constants' bar is wider: their FP32 trajectory is already 3e-6 m from the
# FP64 one after two steps, and the largest gradients (~1e4) move with it.
GRAD_TOL = {"default_constants": 2e-3, "smooth": 1e-3}
# Central-difference steps: the map is strongly nonlinear (larger steps
# disagree with the converged differences by up to 30%); FP64 keeps these
# exact to ~1e-8.
EPS_V = 2e-5
EPS_C = 1e-5
CASES = {"default_constants": (2, True), "smooth": (4, False)}  # name: (steps, default constants)


def scene(lib, default_constants=True):
    p = pbfx.dam_break_params((0.4, 0.4, 0.4), 2, 12 ** 3)
    if not default_constants:
        p.pbf.scorr_enable = 0
        p.pbf.lambda_denom_eps = 1e8
    pos = pbfx.seed_lattice(lib, 12, 12, 12, (0.05, 0.05, 0.05), 0.01, 0.0005, 0xADD, p)
    return p, pos


def grid_density_f64(p, pos, res):
    lo = np.array([p.grid.mins.x, p.grid.mins.y, p.grid.mins.z])
    hi = np.array([p.grid.maxs.x, p.grid.maxs.y, p.grid.maxs.z])
    step = (hi - lo) / res
    ax = [lo[d] + (np.arange(res) + 0.5) * step[d] for d in range(3)]
    gz, gy, gx = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    g = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], 1)
    h2 = float(p.kernel.h) ** 2
    rho = np.zeros(len(g))
    x = np.asarray(pos[:, :3], np.float64)
    for a in range(0, len(x), 256):
        d2 = ((g[:, None, :] - x[None, a:a + 256, :]) ** 2).sum(-1)
        hr2 = np.where(d2 < h2, h2 - d2, 0.0)
        rho += (float(p.particleMass) * float(p.kernel.poly6) * hr2 ** 3).sum(1)
    return rho


def run_f64(orc, p, pos, vel, steps):
    x = np.ascontiguousarray(pos, np.float64)
    v = np.ascontiguousarray(vel, np.float64)
    for _ in range(steps):
        assert orc.oracle_step_f64(C.byref(p), 1, x.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p),
                                   x.shape[0]) == 0
    return x


def loss_f64(orc, p, pos, vel, target, steps):
    x = run_f64(orc, p, pos, vel, steps)
    return float(np.mean((grid_density_f64(p, x, RES) - target) ** 2))


def gpu_gradients(gpu, lib, p, pos, vel, target, steps, every):
    torch = gpu
    n = pos.shape[0]
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.upload(pos, vel)
        tape = C.c_void_p()
        pbfx.check(lib.pbf_forward(s.h, steps, every, C.byref(tape)), "forward")
        try:
            tgt = torch.tensor(target, dtype=torch.float32, device="cuda")
            pbar = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
            vbar = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
            loss = C.c_double()
            pbfx.check(lib.pbf_density_grid_loss(s.h, RES, C.c_void_p(tgt.data_ptr()), C.byref(loss),
                                                 C.c_void_p(pbar.data_ptr())), "loss")
            p0 = torch.zeros_like(pbar)
            v0 = torch.zeros_like(pbar)
            cb = C.c_float()
            torch.cuda.synchronize()
            pbfx.check(lib.pbf_backward(tape, C.c_void_p(pbar.data_ptr()), C.c_void_p(vbar.data_ptr()),
                                        C.c_void_p(p0.data_ptr()), C.c_void_p(v0.data_ptr()), C.byref(cb)),
                       "backward")
            return loss.value, v0.cpu().numpy(), p0.cpu().numpy(), cb.value
        finally:
            lib.pbf_tape_destroy(tape)


@pytest.fixture(scope="module", params=sorted(CASES))
def problem(request, lib, orc):
    steps, default_constants = CASES[request.param]
    p, pos = scene(lib, default_constants)
    rng = np.random.default_rng(7)
    vstar = np.zeros_like(pos)
    vstar[:, :3] = rng.uniform(-0.3, 0.3, (pos.shape[0], 3))
    target = grid_density_f64(p, run_f64(orc, p, pos, vstar, steps), RES)
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.uniform(-0.05, 0.05, (pos.shape[0], 3))
    return p, pos, vel, target, steps, GRAD_TOL[request.param]


@pytest.mark.gpu
def test_velocity_gradient_matches_fp64_central_differences(gpu, lib, orc, problem):
    p, pos, vel, target, steps, tol = problem
    loss, gv, _, _ = gpu_gradients(gpu, lib, p, pos, vel, target, steps, every=3)
    assert loss == pytest.approx(loss_f64(orc, p, pos, vel, target, steps), rel=1e-3)
    rng = np.random.default_rng(3)
    # 64 coordinates, as the benchmark spec's check asks: 56 random and the 8 the
    # loss depends on most
    coords = [(int(i), int(a)) for i, a in zip(rng.integers(0, pos.shape[0], 56), rng.integers(0, 3, 56))]
    # also the particles the loss depends on most
    top = np.argsort(-np.abs(gv[:, :3]).max(1))[:8]
    coords += [(int(i), int(np.argmax(np.abs(gv[i, :3])))) for i in top]
    eps = EPS_V
    g_fd, g_ad = [], []
    for i, a in coords:
        vp, vm = vel.copy(), vel.copy()
        vp[i, a] += eps
        vm[i, a] -= eps
        g_fd.append((loss_f64(orc, p, pos, vp, target, steps) - loss_f64(orc, p, pos, vm, target, steps)) / (2 * eps))
        g_ad.append(float(gv[i, a]))
    g_fd, g_ad = np.array(g_fd), np.array(g_ad)
    scale = np.max(np.abs(g_fd))
    assert scale > 0
    err = np.max(np.abs(g_ad - g_fd)) / scale
    assert err < tol, "max |g - g_fd| / max|g_fd| = %.3e\nad %s\nfd %s" % (err, g_ad, g_fd)


@pytest.mark.gpu
def test_xsph_gradient_matches_fp64_central_differences(gpu, lib, orc, problem):
    p, pos, vel, target, steps, tol = problem
    _, _, _, gc = gpu_gradients(gpu, lib, p, pos, vel, target, steps, every=1)
    eps = EPS_C
    q = pbfx.SimParams.from_buffer_copy(p)
    q.xsph_c = p.xsph_c + eps
    lp = loss_f64(orc, q, pos, vel, target, steps)
    q.xsph_c = p.xsph_c - eps
    lm = loss_f64(orc, q, pos, vel, target, steps)
    fd = (lp - lm) / (2 * eps)
    assert abs(gc - fd) <= tol * abs(fd) + 1e-12, (gc, fd)


@pytest.mark.gpu
def test_checkpoint_interval_does_not_change_gradients(gpu, lib, problem):
    p, pos, vel, target, steps, tol = problem
    ref = gpu_gradients(gpu, lib, p, pos, vel, target, steps, every=steps)
    for every in (1, 3):
        got = gpu_gradients(gpu, lib, p, pos, vel, target, steps, every=every)
        assert got[0] == pytest.approx(ref[0], rel=1e-5)  # grid density uses float atomics
        for a, b in zip(got[1:3], ref[1:3]):
            np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-6 * np.abs(b).max())
        assert got[3] == pytest.approx(ref[3], rel=1e-4)


@pytest.mark.gpu
def test_backward_is_deterministic(gpu, lib, problem):
    """Every particle gathers its terms (no atomics, XSPH gate off): two
    backward passes over the same tape and loss gradient give the same bits."""
    torch = gpu
    p, pos, vel, target, steps, _ = problem
    n = pos.shape[0]
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.upload(pos, vel)
        tape = C.c_void_p()
        pbfx.check(lib.pbf_forward(s.h, steps, 1, C.byref(tape)), "forward")
        try:
            tgt = torch.tensor(target, dtype=torch.float32, device="cuda")
            pbar = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
            vbar = torch.zeros_like(pbar)
            loss = C.c_double()
            pbfx.check(lib.pbf_density_grid_loss(s.h, RES, C.c_void_p(tgt.data_ptr()), C.byref(loss),
                                                 C.c_void_p(pbar.data_ptr())), "loss")
            out = []
            for _ in range(2):
                p0, v0 = torch.zeros_like(pbar), torch.zeros_like(pbar)
                cb = C.c_float()
                pbfx.check(lib.pbf_backward(tape, C.c_void_p(pbar.data_ptr()), C.c_void_p(vbar.data_ptr()),
                                            C.c_void_p(p0.data_ptr()), C.c_void_p(v0.data_ptr()), C.byref(cb)),
                           "backward")
                out.append((p0.cpu().numpy(), v0.cpu().numpy(), cb.value))
        finally:
            lib.pbf_tape_destroy(tape)
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
    assert np.abs(out[0][1]).max() > 0


def test_adjoint_rejects_bad_arguments(lib):
    t = C.c_void_p()
    assert lib.pbf_forward(None, 4, 2, C.byref(t)) == pbfx.PBF_ERR_INVALID
    assert lib.pbf_backward(None, None, None, None, None, None) == pbfx.PBF_ERR_INVALID
    assert lib.pbf_tape_destroy(None) == pbfx.PBF_OK
