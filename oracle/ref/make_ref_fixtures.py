"""Golden fixtures from the reference's own CUDA kernels (run on a GPU).

TEST INFRASTRUCTURE ONLY.  Drives the reference kernels (device images built
by oracle/ref/build_ref.py from the reference sources, launched by
oracle/ref/ref_harness.cu in the reference phase order) on seeded scenes and
stores, per case, the input state and the reference's outputs of ONE step:
sorted keys, permutation, cell tables, lambda of the last iteration, new
positions and velocities.  tests/test_reference_fixtures.py checks the CPU
oracle against them (pinning it), and the GPU tests check the fused step.

Usage (on a machine with a GPU and the built harness):
    python oracle/ref/make_ref_fixtures.py OUT_DIR
then copy OUT_DIR/ref_*.npz into tests/golden/.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "cuda-pbf-fluid-sim_gb300"))
sys.path.insert(0, ROOT)

import pbfx  # noqa: E402


def cases(lib, ref):
    """(name, params, hashed, pos, vel) with states reached by the reference
    itself (lattice start and after k reference steps)."""
    out = []
    for edge, box in ((16, 1.0), (20, 0.6)):
        n = edge ** 3
        for iters in (2,):
            p = pbfx.dam_break_params((box, box, box), iters, n)
            pos = pbfx.seed_lattice(lib, edge, edge, edge, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
            vel = np.zeros_like(pos)
            for hashed in (True, False):
                out.append(("e%d_step0_%s" % (edge, "hashed" if hashed else "dense"), p, hashed, pos.copy(), vel.copy()))
            # advance with the reference to a compressed state
            pa, va = pos.copy(), vel.copy()
            for k in range(30):
                pbfx.ref_step(ref, p, True, pa, va, trace=False)
            for hashed in (True, False):
                out.append(("e%d_step30_%s" % (edge, "hashed" if hashed else "dense"), p, hashed, pa.copy(), va.copy()))
            # neighbour cap engaged, restitution and 1 iteration
            pc = pbfx.dam_break_params((box, box, box), 1, n)
            pc.maxNeighbors = 8
            pc.boundaryRestitution = 0.5
            out.append(("e%d_step30_cap8_iter1" % edge, pc, True, pa.copy(), va.copy()))
    return out


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    lib = pbfx.load()
    ref = pbfx.load_ref()
    if ref is None:
        raise SystemExit("reference device images not present")
    for name, p, hashed, pos, vel in cases(lib, ref):
        pin, vin = pos.copy(), vel.copy()
        tr = pbfx.ref_step(ref, p, hashed, pos, vel, trace=True)
        arrays = {"pos_in": pin, "vel_in": vin, "pos_out": pos, "vel_out": vel,
                  "keys_sorted": tr["keys_sorted"], "perm": tr["perm"], "lambda": tr["lambda"],
                  "params": np.frombuffer(bytes(p), dtype=np.uint8), "hashed": np.int32(hashed)}
        if hashed:
            arrays["unique_keys"] = tr["unique_keys"]
            arrays["offsets"] = tr["offsets"]
        else:
            arrays["cell_start"] = tr["cell_start"]
            arrays["cell_end"] = tr["cell_end"]
        np.savez_compressed(os.path.join(out_dir, "ref_%s.npz" % name), **arrays)
        print("wrote", name, pos.shape[0])


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden"))
