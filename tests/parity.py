"""Parity bars used by the tests (relative errors: |a-b| / max(|b|, floor),
floor = 1% of max|b| unless stated).

GPU (libpbf_gb300) vs the reference's own CUDA kernels: bit-exact.  The
kernels evaluate the reference's expressions in the reference's order with
the same FMA contraction, sqrt, division and powf, so every integer AND
floating-point output is identical (checked against committed fixtures of the
reference kernels and live against the reference kernels on the GPU).

GPU vs the CPU oracle:
  * hash keys, sort permutation, dense and compact cell tables: bit-exact;
  * lambda and XSPH per phase: bit-exact (the oracle spells out the reference
    kernels' FMA contractions);
  * position correction per phase: PHASE_DELTA, normwise - the oracle's
    s_corr exponent is the C library's powf, CUDA's powf is not correctly
    rounded, so a few terms differ by an ulp;
  * state after a full step: STEP_POS for positions (they differ by at most
    1-2 ulps); velocities through the displacement they encode,
    |v_a - v_b| * dt <= STEP_POS * max|x| (v = (x - p) / dt turns one
    position ulp into 1/dt = 120 ulps of velocity); the last iteration's
    lambda normwise (floor = max|lambda|) at STEP_LAMBDA per iteration after
    the first (the ulps compound), because those ulps pass through the next
    solver iteration of the reference's ill-conditioned
    displacement step (a sum of large cancelling terms that is then clamped
    to 0.05 h) and lambda = -C/denom with C = rho/rho0 - 1 near zero for many
    particles.
"""
import numpy as np

PHASE_DELTA = 1e-5  # normwise (floor = max|b|)
STEP_POS = 1e-5
STEP_LAMBDA = 1e-5  # normwise (floor = max|b|), per iteration after the first
STEP_LAMBDA_FLOOR = 1.0


def step_lambda_tol(iters):
    return STEP_LAMBDA * max(1, iters - 1)


def assert_velocities_close(v_a, v_b, pos_b, dt):
    err = float(np.max(np.abs(np.float64(v_a[:, :3]) - np.float64(v_b[:, :3])))) * float(dt)
    scale = float(np.max(np.abs(pos_b[:, :3])))
    if not err <= STEP_POS * scale:
        raise AssertionError("velocities: |dv|*dt = %.3e > %.1e * max|x| (%.3e)" % (err, STEP_POS, STEP_POS * scale))
