"""The adjoint's vector-Jacobian products against an FP64 reference tape.

pbf_backward differentiates the recorded steps in reverse (neighbour sets
held fixed within a step, clamps passing the derivative of the branch
taken).  The reference here is the oracle step run on dual numbers
(oracle_step_jvp) with FP32 values and FP64 derivatives: the values follow
the FP32 trajectory the GPU computes (the FP32 oracle's arithmetic, checked
bit-identical below), and beside them it carries the directional derivative
of that step in FP64, through the same branches.  For cotangents (pbar, vbar)
of the final state and a unit direction e_k of the initial state (one
position or velocity coordinate, or xsph_c), the adjoint's k-th gradient
entry must equal pbar . dx_T + vbar . dv_T of the forward derivative.

Unlike differences of a rollout, this is well conditioned at the reference's
default constants (s_corr on, the displacement clamp engaged for most
particles): C1-size scenes (32,768 particles), one and three steps from a
state 10 steps into the dam break, 49 position and 49 velocity coordinates
(40 random, 9 of the largest entries) and xsph_c, held to 1e-3 of the
largest checked entry.  (With FP64 values the tape would follow the FP64
trajectory, which leaves the FP32 one by ~3e-7 m per step in this chaotic
regime; its derivatives then differ from the FP32 step's by ~1e-3 after one
step and by tens of percent after three.)
"""
import ctypes as C

import numpy as np
import pytest

import pbfx

VJP_TOL = 1e-3  # max |g_adjoint - g_fp64| / max |g_fp64| over the checked entries


def c1_state(lib, orc):
    p = pbfx.dam_break_params((1.0, 1.0, 1.0), 2, 32 ** 3)
    pos = pbfx.seed_lattice(lib, 32, 32, 32, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    vel = np.zeros_like(pos)
    for _ in range(10):
        pbfx.oracle_step(orc, p, True, pos, vel, trace=False)
    return p, pos, vel


def adjoint(gpu, lib, p, pos, vel, pbar, vbar, steps):
    torch = gpu
    with pbfx.Sim(lib, p, hashed=True) as s:
        s.upload(pos, vel)
        s.step(1)  # graph capture, then back to the recorded state
        s.upload(pos, vel)
        tape = C.c_void_p()
        pbfx.check(lib.pbf_forward(s.h, steps, 1, C.byref(tape)), "forward")
        try:
            pb = torch.from_numpy(pbar).cuda()
            vb = torch.from_numpy(vbar).cuda()
            g_pos, g_vel = torch.zeros_like(pb), torch.zeros_like(pb)
            gc = C.c_float()
            pbfx.check(lib.pbf_backward(tape, C.c_void_p(pb.data_ptr()), C.c_void_p(vb.data_ptr()),
                                        C.c_void_p(g_pos.data_ptr()), C.c_void_p(g_vel.data_ptr()), C.byref(gc)),
                       "backward")
            torch.cuda.synchronize()
            return g_pos.cpu().numpy(), g_vel.cpu().numpy(), gc.value
        finally:
            lib.pbf_tape_destroy(tape)


def fp64_directional(orc, p, pos, vel, pbar, vbar, steps, which, i=0, a=0):
    """pbar . dx_T + vbar . dv_T along the FP32 trajectory, for the unit
    direction: which = 'pos' / 'vel' (coordinate a of particle i) or
    'xsph_c'."""
    x = np.ascontiguousarray(pos, np.float64)
    v = np.ascontiguousarray(vel, np.float64)
    dx, dv = np.zeros_like(x), np.zeros_like(v)
    dc = 0.0
    if which == "pos":
        dx[i, a] = 1.0
    elif which == "vel":
        dv[i, a] = 1.0
    else:
        dc = 1.0
    rc = orc.oracle_step_jvp(C.byref(p), 1, 1, pbfx.ptr(x), pbfx.ptr(v), pbfx.ptr(dx), pbfx.ptr(dv), dc,
                             x.shape[0], steps)
    assert rc == 0
    return float(np.sum(pbar[:, :3] * dx[:, :3]) + np.sum(vbar[:, :3] * dv[:, :3]))


@pytest.mark.parametrize("fp32_values", [1, 0])
def test_dual_step_values_are_the_oracle_steps(lib, orc, fp32_values):
    """The dual-number step's value part is the FP32 oracle step (fp32_values
    = 1) or the FP64 oracle step (0), bit for bit, over two steps."""
    p, pos, vel = c1_state(lib, orc)
    x, v = np.ascontiguousarray(pos, np.float64), np.ascontiguousarray(vel, np.float64)
    dx, dv = np.zeros_like(x), np.zeros_like(v)
    assert orc.oracle_step_jvp(C.byref(p), 1, fp32_values, pbfx.ptr(x), pbfx.ptr(v), pbfx.ptr(dx), pbfx.ptr(dv),
                               0.0, x.shape[0], 2) == 0
    if fp32_values:
        x2, v2 = pos.copy(), vel.copy()
        for _ in range(2):
            pbfx.oracle_step(orc, p, True, x2, v2, trace=False)
        np.testing.assert_array_equal(x.astype(np.float32), x2)
        np.testing.assert_array_equal(v.astype(np.float32), v2)
    else:
        x2, v2 = np.ascontiguousarray(pos, np.float64), np.ascontiguousarray(vel, np.float64)
        for _ in range(2):
            assert orc.oracle_step_f64(C.byref(p), 1, pbfx.ptr(x2), pbfx.ptr(v2), x2.shape[0]) == 0
        np.testing.assert_array_equal(x, x2)
        np.testing.assert_array_equal(v, v2)
    assert not dx.any() and not dv.any()


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [1, 3])
def test_adjoint_vjp_matches_fp64_forward_derivative(gpu, lib, orc, steps):
    p, pos, vel = c1_state(lib, orc)
    n = pos.shape[0]
    rng = np.random.default_rng(11 + steps)
    pbar = np.zeros((n, 4), np.float32)
    vbar = np.zeros((n, 4), np.float32)
    pbar[:, :3] = rng.normal(size=(n, 3))
    vbar[:, :3] = rng.normal(size=(n, 3)) * float(p.dt)  # velocities are (x - p)/dt: comparable weight
    g_pos, g_vel, g_c = adjoint(gpu, lib, p, pos, vel, pbar, vbar, steps)
    got, want = [], []
    for which, g in (("pos", g_pos), ("vel", g_vel)):
        picks = [(int(i), int(a)) for i, a in zip(rng.integers(0, n, 40), rng.integers(0, 3, 40))]
        top = np.argsort(-np.abs(g[:, :3]).max(1))[:9]  # and the largest entries
        picks += [(int(i), int(np.argmax(np.abs(g[i, :3])))) for i in top]
        for i, a in picks:
            got.append(float(g[i, a]))
            want.append(fp64_directional(orc, p, pos, vel, pbar, vbar, steps, which, i, a))
    got.append(float(g_c))
    want.append(fp64_directional(orc, p, pos, vel, pbar, vbar, steps, "xsph_c"))
    got, want = np.array(got), np.array(want)
    scale = np.max(np.abs(want))
    assert scale > 0
    err = np.max(np.abs(got - want)) / scale
    assert err < VJP_TOL, "max |g - g64| / max |g64| = %.3e\nadjoint %s\nfp64 %s" % (err, got, want)
    # xsph_c on its own scale
    assert abs(got[-1] - want[-1]) <= VJP_TOL * abs(want[-1]) + 1e-9 * scale, (got[-1], want[-1])
