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
    1-2 ulps); STEP_VEL for velocities, normwise: v = (x - p) / dt turns a
    position ulp into 1/dt = 120 ulps of an O(1) quantity, so slow particles
    are compared against the velocity scale; STEP_LAMBDA for the last
    iteration's lambda, because the ulps pass through the next solver
    iteration of the reference's ill-conditioned displacement step (a sum of
    large cancelling terms that is then clamped to 0.05 h).
"""

PHASE_DELTA = 1e-5  # normwise (floor = max|b|)
STEP_POS = 1e-5
STEP_VEL = 1e-5  # normwise (floor = max|b|)
STEP_VEL_FLOOR = 1.0
STEP_LAMBDA = 1e-4
