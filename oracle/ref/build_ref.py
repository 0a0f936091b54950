"""Builds device images of the reference's own CUDA kernels (test checker).

TEST INFRASTRUCTURE ONLY.  Compiles the reference sources where they lie
(/root/reference/sim/*.cu, read-only; nothing is copied) into sm_103a cubins
under oracle/_ref/, which is git-ignored.  Device code only: the host side is
oracle/ref/ref_harness.cu, which loads these images with the CUDA driver API
and launches the kernels in the reference phase order.

Run where the reference sources exist:  python oracle/ref/build_ref.py
[REFERENCE_ROOT].  The reference checkout is the argument, else the
PBF_REFERENCE_ROOT environment variable, else /root/reference.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
DEFAULT_REFERENCE_ROOT = "/root/reference"


def reference_root(argv=None) -> str:
    """The reference checkout: argument, then $PBF_REFERENCE_ROOT, then the default."""
    if argv:
        return argv[0]
    return os.environ.get("PBF_REFERENCE_ROOT", DEFAULT_REFERENCE_ROOT)


SRC = os.path.join(reference_root(sys.argv[1:] if __name__ == "__main__" else None), "sim")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
# The kernels of the step (sim/phases.cpp, sim/post_ops.cpp).  The build
# mirrors the reference's: no fast-math, default FMA contraction.
UNITS = ["integrate", "boundary", "hash_keys", "cell_ranges", "cell_compact", "pbf_lambda", "pbf_delta_apply",
         "xsph"]


def build_one(name):
    src = os.path.join(SRC, name + ".cu")
    out = os.path.join(OUT, name + ".cubin")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cmd = [NVCC, "-std=c++17", "-O3", "-arch=sm_103a", "-cubin", "-I", SRC, src, "-o", out + ".tmp"]
    if name == "pbf_lambda":
        cmd[1:1] = ["-include", os.path.join(HERE, "ref_globals_shim.cuh")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference kernel build failed: %s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(out + ".tmp", out)
    return out


def main():
    if not os.path.isdir(SRC):
        print("reference sources not present; nothing to build")
        return 0
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=8) as ex:
        outs = list(ex.map(build_one, UNITS))
    print("built", len(outs), "reference device images in", OUT)
    return 0


if __name__ == "__main__":
    sys.exit(main())
