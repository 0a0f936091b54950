"""bench.py's reference arm on CPU (no GPU needed): the JSON line's contract
keys on the 32,768-particle case, the 'unavailable' lines of the workloads the
reference has no counterpart for, and the rank rule (rank 0 alone prints)."""
import contextlib
import io
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def run_main(argv):
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        rc = bench.main(argv)
    lines = [ln for ln in out.getvalue().splitlines() if ln.startswith("{")]
    return rc, lines


def test_reference_arm_line():
    rc, lines = run_main(["--impl", "reference", "--config", "c1", "--steps", "2", "--warmup", "3"])
    assert rc == 0 and len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "impl", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["particles"] == 32768


@pytest.mark.parametrize("config", ["c4", "c5"])
def test_reference_arm_unavailable(config):
    rc, lines = run_main(["--impl", "reference", "--config", config, "--steps", "1", "--warmup", "3"])
    assert rc == 0 and len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unavailable"]


def test_reference_arm_other_ranks_print_nothing():
    args = bench.argparse.Namespace(steps=1, warmup=3, ref_budget=1.0)
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        assert bench.run_reference(args, bench.CONFIGS["c1"], 2, 1) == 0
    assert out.getvalue() == ""


def test_warmup_floor():
    with pytest.raises(SystemExit):
        bench.main(["--warmup", "2"])


def test_reference_arm_config_is_ours():
    """Both arms describe the workload with the same config object."""
    rc, lines = run_main(["--impl", "reference", "--config", "c1", "--steps", "2", "--warmup", "3"])
    d = json.loads(lines[0])
    args = bench.argparse.Namespace(steps=2, warmup=3)
    import pbfx

    orc = pbfx.load_oracle()
    p, pos, _ = bench.scene(None, bench.CONFIGS["c1"], orc=orc)
    assert d["config"] == bench.config_record(bench.CONFIGS["c1"], pos.shape[0], pbfx.num_cells(p), 1, args)


def test_reference_arm_loads_no_product_library(built):
    """The CPU arm runs the oracle alone: the product library is never mapped."""
    import subprocess

    code = ("import sys, io, contextlib; sys.path.insert(0, %r); import bench\n"
            "with contextlib.redirect_stdout(io.StringIO()):\n"
            "    bench.main(['--impl', 'reference', '--config', 'c1', '--steps', '1', '--warmup', '3'])\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('product' if 'libpbf_gb300' in maps else 'clean', 'oracle' if 'liboracle' in maps else '')\n"
            % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["clean", "oracle"], r.stdout


@pytest.mark.parametrize("config", ["c1", "c2"])
def test_oracle_scene_generation_matches_library(lib, orc, config):
    """The oracle's restated scene generation gives the library's bits."""
    import ctypes as C

    cfg = bench.CONFIGS[config]
    p_lib, pos_lib, _ = bench.scene(lib, cfg)
    p_orc, pos_orc, _ = bench.scene(None, cfg, orc=orc)
    assert bytes(p_lib) == bytes(p_orc)
    assert C.sizeof(p_lib) == C.sizeof(p_orc)
    assert pos_lib.tobytes() == pos_orc.tobytes()


def test_committed_step_profile_feeds_the_c2_line():
    """The C2 line's DRAM traffic and issue roofline come from the committed
    ncu figures of one step of its window (profiles/c2_dram_traffic.txt)."""
    cap = bench.read_traffic(bench.CONFIGS["c2"], bench.argparse.Namespace(config="c2", steps=20, warmup=5))
    assert cap is not None and 5 <= cap["step"] < 25
    for phase in ("lists_1", "lambda_1", "delta_1", "lambda_2", "delta_2", "commit"):
        dram, inst = cap["phases"][phase]
        assert dram > 0 and inst > 0
    assert bench.read_traffic(bench.CONFIGS["c3"], bench.argparse.Namespace(config="c3", steps=30, warmup=20)) is None


def test_dominant_kernel_counts_every_launch():
    """The roofline's kernel is the one with the most time over all its
    launches in a step, not the longest single launch."""
    ph = {"predict_keys": 0.011, "sort": 0.075, "lists_1": 0.238, "lambda_1": 0.116, "delta_1": 0.177,
          "lambda_2": 0.116, "delta_2": 0.182, "commit": 0.143}
    dom, members, ms = bench.dominant_kernel(ph)
    assert dom == "delta" and members == ["delta_1", "delta_2"] and abs(ms - 0.359) < 1e-9
    dom, members, ms = bench.dominant_kernel({"lists_1": 0.3, "delta_1": 0.2, "commit": 0.1})
    assert dom == "lists" and members == ["lists_1"]
