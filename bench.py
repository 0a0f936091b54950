"""Benchmark of the GB300 PBF step (one JSON line on stdout).

Workload (default): the 1,048,576-particle dam break - a 128x64x128 jittered
lattice (spacing 0.01, jitter +-0.0005 from mt19937_64(0xC0FFEE)) in the
[0,2]x[0,1]x[0,2] box, h = 2.5r, 2 solver iterations, hashed grid.  A "step"
is one full simulation step of all particles.  W warm-up steps from the
seeded lattice, then K timed steps; L2 is flushed (256 MiB write) before every
timed step and each step is timed with CUDA events on the simulator's stream.

  value      particle-steps/s, state resident in HBM
  e2e        the same through pbf_step_host: pinned host pos/vel copied in,
             one step, copied back, every step (wall clock), over the same
             steps as the timed region (restarted from its first state)
  roofline   dominant kernel of the step, the one with the most time over
             its launches (from a live per-phase profile): algorithmic bytes
             per launch / its CUDA-event time per launch, vs the measured HBM
             copy bandwidth
  cpu_baseline  the CPU oracle (OpenMP, all host threads) on a bounded
             sample of the same workload (rank 0, N = 1)

--impl reference times the reference arm: the reference has no CPU PBF path
(sim/kernel_fallback.cpp is a vector add), so its CPU implementation is the
restatement in oracle/, run on all host threads.

Multi-GPU: the path does not shard (a single scene needs halo exchanges), so
--gpus N runs N independent replicas ("scaling": "weak"); value = all ranks'
particle-steps / the slowest rank's timed region.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cuda-pbf-fluid-sim_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, ROOT)

CONFIGS = {
    # name: box, lattice, solver iters, grid, second block (lattice, origin seed)
    "c1": dict(box=(1.0, 1.0, 1.0), lattice=(32, 32, 32), iters=2, hashed=True,
               workload="dam_break_32k_2iter_hashed (32x32x32 lattice, [0,1]^3 box)"),
    "c2": dict(box=(2.0, 1.0, 2.0), lattice=(128, 64, 128), iters=2, hashed=True,
               workload="dam_break_1M_2iter_hashed (128x64x128 lattice, [0,2]x[0,1]x[0,2] box)"),
    "c2_dense": dict(box=(2.0, 1.0, 2.0), lattice=(128, 64, 128), iters=2, hashed=False,
                     workload="dam_break_1M_2iter_dense (128x64x128 lattice, [0,2]x[0,1]x[0,2] box)"),
    # adjoint: 32 scenes of a 64^3 lattice in a 1 m box, 60 steps, checkpoints every 10
    # 8.4M-particle slab plus a 1M block dropped 0.5 m above it (x, z seeded),
    # 4 iterations; the box is 2.5 m high so the second block fits
    "c3": dict(box=(3.0, 2.5, 3.0), lattice=(256, 128, 256), iters=4, hashed=True, drop=(128, 64, 128, 0.5),
               list_capacity=1024, metric="particle-steps/s @9.4M",
               workload="dam_break_9.4M_4iter_hashed (256x128x256 lattice + 128x64x128 block 0.5 m above, "
                        "[0,3]x[0,2.5]x[0,3] box)"),
    "c3_dense": dict(box=(3.0, 2.5, 3.0), lattice=(256, 128, 256), iters=4, hashed=False, drop=(128, 64, 128, 0.5),
                     list_capacity=1024, metric="particle-steps/s @9.4M",
                     workload="dam_break_9.4M_4iter_dense (256x128x256 lattice + 128x64x128 block 0.5 m above, "
                              "[0,3]x[0,2.5]x[0,3] box)"),
    # (65,536 particles per scene: a 64x32x32 lattice; a 64^3 one would hold 262,144)
    "c5": dict(adjoint=True, scenes=32, lattice=(64, 32, 32), box=(1.0, 1.0, 1.0), iters=2, hashed=True,
               horizon=60, every=10, res=32,
               workload="adjoint_32x65536 (64x32x32 lattices in [0,1]^3, 2 iterations, 60 steps, checkpoints every "
                        "10, loss on the SPH density at 32^3 grid points)"),
    # batched ensemble: 256 seeded scenes (pbfx.ensemble_scenes)
    "c4": dict(scenes=256, seed=0xE45E, iters=3, hashed=True,
               workload="ensemble_256_scenes (N_s log-uniform in [2048, 65536], boxes U[0.3,1]^3 m, gravity tilted "
                        "<= 15 deg, 2 or 3 iterations, seed 0xE45E)"),
}

METRIC = "particle-steps/s @1M"
UNIT = "particle-steps/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def key_bits(num_cells: int) -> int:
    return max(1, int(num_cells - 1).bit_length())


def alg_bytes_per_particle(phase: str, n: int, num_cells: int, hashed: bool, iters: int) -> float:
    """Compulsory bytes per particle of one launch of each phase (neighbour
    gathers counted once; float4 state, u32 keys/ids)."""
    passes = (key_bits(num_cells) + 7) // 8
    table = 4.0 * (num_cells + 1) / max(n, 1)
    if phase == "predict_keys":
        return 16 + 16 + 4  # R pos, vel; W key
    if phase == "sort":
        return 4 + 4 + 8 + 16 * (passes - 1)  # histogram read, first pass R key W pair, then R/W pairs
    if phase == "gather_tables":
        return 4 + 16 + 16 + 16 + 16 + 4 + table + (12 if hashed else 0)
    if phase.startswith("lambda"):
        return 16 + 4 + 4  # R pred, key; W lambda (table reads shared by a cell)
    if phase.startswith("delta"):
        last = phase == "delta_%d" % iters
        return 16 + 4 + 4 + 16 + (32 if last else 0)  # R pred, lambda, key; W pred (+ R pos_s, W vel)
    if phase == "commit":
        return 16 + 16 + 4 + 4 + 16 + 16  # R pred, vel_s, key, perm; W pos, vel
    if phase.startswith("lists"):
        return 16 + 4  # R pred, key (the lists themselves are not algorithmic traffic)
    return 0.0


def dominant_kernel(phase_ms: dict):
    """The kernel with the most time per step over all its launches (phases
    lambda_1 and lambda_2 are two launches of one kernel): (kernel, its
    phases, its ms per step)."""
    fam_of = {k: (k.rsplit("_", 1)[0] if k.rsplit("_", 1)[-1].isdigit() else k) for k in phase_ms}
    per_step = {}
    for k, f in fam_of.items():
        per_step[f] = per_step.get(f, 0.0) + phase_ms[k]
    dom = max(per_step, key=per_step.get)
    return dom, [k for k in phase_ms if fam_of[k] == dom], per_step[dom]


def tuning_report(lib, chosen, ms, steps, api):
    """The autotuner's choice and the per-shape step times it measured."""
    import pbfx
    shapes = pbfx.tile_shapes(lib)
    return {"shape": chosen, "tile": shapes[chosen][0], "stage_slots": shapes[chosen][1],
            "ms_per_step": {"%d/%d" % sh: round(m, 4) for sh, m in zip(shapes, ms)},
            "what": "%s: every tile shape (particles per CTA / staged slots) timed over %d steps from the "
                    "post-warm-up state, state restored, untimed" % (api, steps)}


def issue_peak(clk) -> float:
    """Warp instructions per second the GPU can issue: 4 schedulers per SM."""
    import torch

    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    return 4.0 * sms * mhz * 1e6


def step_alg_bytes(num_cells: int, iters: int) -> float:
    """Whole-step compulsory bytes: 202 + 16 P + 60 iters per particle."""
    passes = (key_bits(num_cells) + 7) // 8
    return 202 + 16 * passes + 60 * iters


class ClockSampler:
    FIELDS = ("index,pci.bus_id,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, bus_id: str | None):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            rows.append(parts)
        os.unlink(self.path)
        if bus_id:
            mine = [r for r in rows if r[1].lower().endswith(bus_id.lower()[-12:])]
            rows = mine or rows
        if not rows:
            return None
        sm = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        mx = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        reasons = set()
        for r in rows:
            for name, col in (("hw_slowdown", 6), ("hw_thermal_slowdown", 7), ("sw_thermal_slowdown", 8),
                              ("sw_power_cap", 9)):
                if r[col].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if os.environ.get("PBF_BENCH_BACKEND", "") != "gloo" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def aggregate(local_seconds: float, local_units: float, world: int):
    """Max of the timed region over ranks and sum of processed units."""
    if world <= 1:
        return local_seconds, local_units
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([local_seconds], dtype=torch.float64, device=dev)
    u = torch.tensor([local_units], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def scene(lib, cfg, orc=None):
    """(params, pos, vel) of a configuration.  With orc given, the oracle's
    restatement of the scene generation is used instead of the library's
    (the CPU reference arm loads no product code); both give the same bits."""
    import pbfx

    if orc is not None:
        params_of = lambda box, iters, n: pbfx.oracle_dam_break_params(orc, box, iters, n)  # noqa: E731
        lattice = lambda *a: pbfx.oracle_seed_lattice(orc, *a)  # noqa: E731
    else:
        params_of = pbfx.dam_break_params
        lattice = lambda *a: pbfx.seed_lattice(lib, *a)  # noqa: E731
    nx, ny, nz = cfg["lattice"]
    n = nx * ny * nz
    p = params_of(cfg["box"], cfg["iters"], n)
    pos = lattice(nx, ny, nz, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    if "drop" in cfg:
        # a second block, its bottom `gap` above the first block's top, at a
        # seeded (x, z) inside the box
        bx, by, bz, gap = cfg["drop"]
        rng = np.random.default_rng(0xD209)
        ox = 0.005 + rng.uniform(0.0, cfg["box"][0] - 0.01 * bx - 0.01)
        oz = 0.005 + rng.uniform(0.0, cfg["box"][2] - 0.01 * bz - 0.01)
        oy = 0.005 + 0.01 * ny + gap
        q = params_of(cfg["box"], cfg["iters"], n + bx * by * bz)
        pos2 = lattice(bx, by, bz, (ox, oy, oz), 0.01, 0.0005, 0xC0FFEE + 1, q)
        pos = np.ascontiguousarray(np.concatenate([pos, pos2]))
        p = q
    return p, pos, np.zeros_like(pos)


def config_record(cfg, n: int, nc: int, world: int, args) -> dict:
    """The line's config object, shared by both arms so that they describe
    the same workload in the same words."""
    return {"workload": cfg["workload"], "particles": n, "solver_iters": cfg["iters"], "cells": nc,
            "grid": "hashed" if cfg["hashed"] else "dense", "parallelism": "replicas" if world > 1 else "single",
            "timed_steps": "steps %d..%d of the run from the seeded lattice" % (args.warmup,
                                                                              args.warmup + args.steps - 1),
            "l2": "flushed before every timed step (256 MiB write, untimed)",
            "arithmetic": getattr(args, "math", "exact")}


def cpu_rate(orc, p, hashed, pos, vel, budget_s: float, max_steps: int):
    """Oracle steps from (pos, vel) until the budget is used; returns
    (particle-steps/s, steps, seconds)."""
    import pbfx

    pos, vel = pos.copy(), vel.copy()
    n = pos.shape[0]
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        pbfx.oracle_step(orc, p, hashed, pos, vel, trace=False)
        steps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return n * steps / dt, steps, dt


def launcher_path(lib, p, pos0, hashed: bool, warmup: int, steps: int):
    """The step through the reference-layout phase launchers (pbf_launch_*,
    include/pbf/pbf.h), in the reference's phase order (sim/phases.cpp:30-117,
    sim/post_ops.cpp:25-85): what a reference build linked against this
    library runs.  Returns (device ms per step, final positions)."""
    import torch

    import pbfx

    n = pos0.shape[0]
    nc = pbfx.num_cells(p)
    dp = pbfx.device_params(p)
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    f4 = lambda: torch.empty((n, 4), dtype=torch.float32, device="cuda")  # noqa: E731
    u32 = lambda k: torch.empty(max(k, 1), dtype=torch.int32, device="cuda")  # noqa: E731
    pos, pred, delta, vel_old = torch.from_numpy(pos0).cuda(), f4(), f4(), f4()
    vel = torch.zeros_like(pos)
    lam = torch.empty(n, dtype=torch.float32, device="cuda")
    keys, idx, ks, ids = u32(n), u32(n), u32(n), u32(n)
    uk, off, cnt, st, en = u32(n), u32(n + 1), u32(1), u32(nc), u32(nc)
    tb, sb = C.c_size_t(), C.c_size_t()
    pbfx.check(lib.pbf_sort_pairs_query(C.byref(tb), n), "sort query")
    pbfx.check(lib.pbf_cell_compact_scratch_query(C.byref(sb), n), "compact scratch query")
    sort_tmp = torch.empty(max(tb.value, 1), dtype=torch.uint8, device="cuda")
    scratch = torch.empty(max(sb.value, 1), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    S = C.c_void_p(stream.cuda_stream)
    inv_dt = C.c_float(np.float32(1.0) / np.float32(p.dt))
    if hashed:
        tab = (P(uk), P(off), P(cnt))
        lam_fn, delta_fn, xsph_fn = lib.pbf_launch_lambda_compact, lib.pbf_launch_delta_apply_compact, \
            lib.pbf_launch_xsph_compact
    else:
        tab = (P(st), P(en))
        lam_fn, delta_fn, xsph_fn = lib.pbf_launch_lambda, lib.pbf_launch_delta_apply, lib.pbf_launch_xsph

    def step(cur, nxt):
        ck = pbfx.check
        ck(lib.pbf_launch_integrate_pred(P(cur), P(vel), P(nxt), p.gravity, C.c_float(p.dt), n, S))
        ck(lib.pbf_launch_boundary(P(nxt), P(vel), C.byref(p.grid), C.c_float(0.0), n, S))
        ck(lib.pbf_launch_hash_keys(P(keys), P(idx), P(nxt), C.byref(p.grid), n, S))
        ck(lib.pbf_launch_sort_pairs(P(sort_tmp), tb.value, P(keys), P(ks), P(idx), P(ids), n, S))
        if hashed:
            ck(lib.pbf_launch_cell_ranges_compact(P(scratch), sb.value, P(uk), P(off), P(cnt), P(ks), n, S))
        else:
            ck(lib.pbf_launch_cell_ranges(P(st), P(en), P(ks), n, nc, S))
        for _ in range(p.solverIters):
            ck(lam_fn(P(lam), P(nxt), P(ids), P(ks), *tab, C.byref(dp), n, S))
            ck(delta_fn(P(nxt), P(delta), P(lam), P(ids), P(ks), *tab, C.byref(dp), n, S))
        ck(lib.pbf_launch_boundary(P(nxt), P(vel), C.byref(p.grid), C.c_float(0.0), n, S))
        ck(lib.pbf_launch_velocity(P(vel), P(cur), P(nxt), inv_dt, n, S))
        if p.xsph_c > 0.0:
            with torch.cuda.stream(stream):
                vel_old.copy_(vel)
            ck(xsph_fn(P(vel), P(vel_old), P(nxt), P(ids), P(ks), *tab, C.byref(dp), n, S))
        ck(lib.pbf_launch_boundary(P(nxt), P(vel), C.byref(p.grid), C.c_float(p.boundaryRestitution), n, S))

    torch.cuda.synchronize()
    for _ in range(warmup):
        step(pos, pred)
        pos, pred = pred, pos
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        ev[k][0].record(stream)
        step(pos, pred)
        ev[k][1].record(stream)
        pos, pred = pred, pos
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / steps, pos.cpu().numpy()


def run_reference(args, cfg, world, rank):
    if rank != 0:
        return 0
    import __graft_entry__ as g
    import pbfx

    g.build_oracle()  # the CPU restatement only: this arm loads no product library
    orc = pbfx.load_oracle()
    p, pos, vel = scene(None, cfg, orc=orc)
    n = pos.shape[0]
    cores = orc.oracle_num_threads()
    for _ in range(args.warmup):
        pbfx.oracle_step(orc, p, cfg["hashed"], pos, vel, trace=False)
    rate, steps, secs = cpu_rate(orc, p, cfg["hashed"], pos, vel, args.ref_budget, args.steps)
    sample = ("%d of the %d requested steps of the %d-particle workload after %d warm-up steps "
              "(time budget %.0f s)" % (steps, args.steps, n, args.warmup, args.ref_budget))
    line = {
        "metric": cfg.get("metric", METRIC), "value": rate, "unit": UNIT, "impl": "reference", "n_gpus": world,
        "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice, mt19937_64 0xC0FFEE)",
        "config": config_record(cfg, n, pbfx.num_cells(p), world, args),
        "implementation": "CPU restatement of the reference kernels (oracle/pbf_oracle.cpp), OpenMP over "
                          "particles; the reference has no CPU PBF path",
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def read_traffic(cfg, args):
    """The committed ncu figures of one step of the default C2 window:
    {"step": absolute step index, "phases": {phase: (DRAM bytes, warp
    instructions)}}, or None for other workloads."""
    tfile = os.path.join(ROOT, "profiles", "c2_dram_traffic.txt")
    if args.config != "c2" or not os.path.exists(tfile):
        return None
    step, phases = None, {}
    for ln in open(tfile):
        f = ln.split()
        if not f:
            continue
        if f[0] == "#":
            if len(f) >= 3 and f[1] == "step:":
                step = int(f[2])
            continue
        phases[f[0]] = (int(f[1]), int(f[2]))
    return {"step": step, "phases": phases} if step is not None and phases else None


def density_error_report(lib, orc, sim, p, hashed, pos, vel):
    """Density-constraint error of the state after the timed steps: the
    library's statistics (pbf_density_stats: mean |C|, max |C|, mean max(C,0),
    mean neighbours; C = rho/rho0 - 1) against the FP64 oracle's evaluation of
    the same positions, and one more step taken by the library (FP32) and by
    the FP64 oracle from that state, each scored in FP64."""
    import pbfx

    names = ("mean_abs_C", "max_abs_C", "mean_pos_C", "mean_neighbours")
    n = pos.shape[0]
    gpu = sim.density_stats()
    ev = (C.c_double * 4)()
    orc.oracle_density_stats_f32pos(C.byref(p), pbfx.ptr(pos), n, C.byref(ev))
    # one step each: FP32 library, FP64 oracle
    sim.step()
    g1, _ = sim.download()
    s32 = (C.c_double * 4)()
    orc.oracle_density_stats_f32pos(C.byref(p), pbfx.ptr(g1), n, C.byref(s32))
    p64 = np.ascontiguousarray(pos, dtype=np.float64)
    v64 = np.ascontiguousarray(vel, dtype=np.float64)
    t0 = time.perf_counter()
    if orc.oracle_step_f64(C.byref(p), 1 if hashed else 0, pbfx.ptr(p64), pbfx.ptr(v64), n) != 0:
        return None
    t64 = time.perf_counter() - t0
    s64 = (C.c_double * 4)()
    orc.oracle_density_stats_f64pos(C.byref(p), pbfx.ptr(p64), n, C.byref(s64))
    return {
        "state": "after the timed steps",
        "library_fp32": dict(zip(names, list(gpu))),
        "fp64_oracle_same_positions": dict(zip(names, list(ev))),
        "stats_abs_diff_mean_abs_C": abs(gpu[0] - ev[0]),
        "next_step": {"library_fp32": dict(zip(names, list(s32))), "fp64_oracle": dict(zip(names, list(s64))),
                      "abs_diff_mean_abs_C": abs(s32[0] - s64[0]), "fp64_oracle_seconds": t64},
    }


def ensemble_density_error(ens, scenes, orc, sample: int = 8):
    """Density error of the ensemble against FP64, on every (S / sample)-th
    scene: from the state after the timed steps, one ensemble step (FP32) and
    one FP64 oracle step of the scene, each scored in FP64 (mean |C| with
    C = rho/rho0 - 1).  The ensemble is left one step further on."""
    import pbfx

    pos, vel = ens.download()
    ens.step(1)
    g1, _ = ens.download()
    off = ens.offsets.astype(np.int64)
    picks = list(range(0, len(scenes), max(1, len(scenes) // sample)))[:sample]
    rows = []
    for k in picks:
        p = scenes[k]
        a, b = off[k], off[k + 1]
        n = int(b - a)
        s32 = (C.c_double * 4)()
        orc.oracle_density_stats_f32pos(C.byref(p), pbfx.ptr(np.ascontiguousarray(g1[a:b])), n, C.byref(s32))
        p64 = np.ascontiguousarray(pos[a:b], dtype=np.float64)
        v64 = np.ascontiguousarray(vel[a:b], dtype=np.float64)
        if orc.oracle_step_f64(C.byref(p), 1, pbfx.ptr(p64), pbfx.ptr(v64), n) != 0:
            return None
        s64 = (C.c_double * 4)()
        orc.oracle_density_stats_f64pos(C.byref(p), pbfx.ptr(p64), n, C.byref(s64))
        rows.append({"scene": k, "particles": n, "fp32_mean_abs_C": s32[0], "fp64_mean_abs_C": s64[0],
                     "abs_diff": abs(s32[0] - s64[0])})
    return {"state": "one step after the timed steps", "scenes": rows,
            "max_abs_diff_mean_abs_C": max(r["abs_diff"] for r in rows),
            "what": "ensemble step (FP32, GPU) vs FP64 oracle step of the same scene from the same state, both "
                    "scored in FP64"}


def e2e_step_count(args) -> int:
    """Steps of the end-to-end measurement: the timed steps unless capped."""
    return args.steps if args.e2e_steps <= 0 else max(1, min(args.steps, args.e2e_steps))


def run_ours(args, cfg, world, rank, local):
    import torch

    import __graft_entry__ as g
    import pbfx

    if rank == 0 or world == 1:
        g.build_library()
        g.build_oracle()
    barrier(world)
    torch.cuda.set_device(local)
    lib = pbfx.load()
    p, pos, vel = scene(lib, cfg)
    n = pos.shape[0]
    nc = pbfx.num_cells(p)
    hashed = cfg["hashed"]
    hbm_peak, peak_kind = peaks()

    sim = pbfx.Sim(lib, p, hashed=hashed)
    if "list_capacity" in cfg:
        sim.set_list_capacity(cfg["list_capacity"])
    if args.math == "fast":
        sim.set_math_mode(pbfx.PBF_MATH_FAST)
    sim.upload(pos, vel)
    stream = torch.cuda.ExternalStream(sim.stream_ptr())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    pp = C.byref(p)

    for _ in range(args.warmup):
        pbfx.check(lib.pbf_step(sim.h, pp))
    pbfx.check(lib.pbf_synchronize(sim.h))
    tuned = None
    if args.autotune_steps > 0:  # untimed; the tuner puts the state back
        tuned = tuning_report(lib, *sim.autotune(steps=args.autotune_steps, params=p), args.autotune_steps,
                              "pbf_autotune_tile_shape")
    snap_pos, snap_vel = sim.download()  # state at the start of the timed region

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler()
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()  # L2 flush, outside the timed window
            ev[k][0].record(stream)
            lib.pbf_step(sim.h, pp)
            ev[k][1].record(stream)
    pbfx.check(lib.pbf_synchronize(sim.h))
    torch.cuda.synchronize()
    barrier(world)
    bus = None
    try:
        bus = torch.cuda.get_device_properties(local).pci_bus_id  # type: ignore[attr-defined]
    except Exception:
        bus = None
    clk = clocks.stop(bus)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    local_s = sum(step_ms) / 1e3
    total_s, units = aggregate(local_s, float(n) * args.steps, world)
    value = units / total_s

    final_pos, final_vel = sim.download()  # state after the timed steps
    dens = density_error_report(lib, pbfx.load_oracle(), sim, p, hashed, final_pos, final_vel) \
        if rank == 0 and world == 1 and not args.no_cpu_baseline else None

    # Live per-phase profile over the timed window: the state is put back to
    # the window's first step and each of its steps is run once more with an
    # event between phases, so every figure below describes the timed steps.
    sim.upload(snap_pos, snap_vel)
    prof, per_step = {}, []
    for _ in range(args.steps):
        row = sim.profile_step()
        per_step.append(dict(row))
        for name, ms in row:
            prof.setdefault(name, []).append(ms)
    prof_pos, _ = sim.download()
    avg = {k: sum(v) / len(v) for k, v in prof.items()}
    total_phase = sum(avg.values())
    dom, members, dom_step_ms = dominant_kernel(avg)
    dom_ms = dom_step_ms / len(members)
    dom_bytes = sum(alg_bytes_per_particle(k, n, nc, hashed, cfg["iters"]) for k in members) / len(members) * n
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    # DRAM traffic and warp instructions per launch, from the committed ncu
    # capture of one step of the same window (profiles/c2_dram_traffic.txt).
    cap = read_traffic(cfg, args)
    traffic = inst = None
    step_traffic = None
    if cap is not None:
        recs = [cap["phases"].get(k) for k in members]
        if all(recs):
            traffic = sum(r[0] for r in recs) / len(recs)
            inst = sum(r[1] for r in recs) / len(recs)
        if set(avg) <= set(cap["phases"]):
            step_traffic = sum(v[0] for v in cap["phases"].values())

    # End to end through host buffers, from the state the timed region started
    # from (the cost per step changes as the fluid settles).
    e2e_steps = e2e_step_count(args)
    hp = torch.from_numpy(snap_pos.copy()).pin_memory()
    hv = torch.from_numpy(snap_vel.copy()).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        pbfx.check(lib.pbf_step_host(sim.h, pp, C.c_void_p(hp.data_ptr()), C.c_void_p(hv.data_ptr())))
    e2e_s = time.perf_counter() - t0
    e2e_total, e2e_units = aggregate(e2e_s, float(n) * e2e_steps, world)
    e2e_pos, _ = sim.download()
    # The other arithmetic mode over the same window (same state, same L2
    # flushes), for comparison.
    other = "fast" if args.math == "exact" else "exact"
    sim.set_math_mode(pbfx.PBF_MATH_FAST if other == "fast" else pbfx.PBF_MATH_EXACT)
    sim.upload(snap_pos, snap_vel)
    pbfx.check(lib.pbf_step(sim.h, pp))  # graph capture of the other mode, then back to the window's start
    sim.upload(snap_pos, snap_vel)
    torch.cuda.synchronize()
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            ev2[k][0].record(stream)
            lib.pbf_step(sim.h, pp)
            ev2[k][1].record(stream)
    pbfx.check(lib.pbf_synchronize(sim.h))
    torch.cuda.synchronize()
    other_ms = sum(a.elapsed_time(b) for a, b in ev2) / args.steps
    other_pos, _ = sim.download()
    sim.set_math_mode(pbfx.PBF_MATH_FAST if args.math == "fast" else pbfx.PBF_MATH_EXACT)
    launches = sim.launches_per_step() * args.steps
    list_cap, list_longest, list_overflowed = sim.list_stats()
    sim.close()
    cap_step = cap["step"] if cap else None
    cap_k = (cap_step - args.warmup) if cap_step is not None else None
    issue = None
    if inst is not None and cap_k is not None and 0 <= cap_k < args.steps and all(
            k in per_step[cap_k] for k in members):
        t_cap = sum(per_step[cap_k][k] for k in members) / len(members)
        issue = {"kernel": dom, "launches_per_step": len(members), "step": cap_step, "unit": "warp-instructions/s",
                 "warp_instructions_per_launch": inst, "ms_at_step": t_cap,
                 "achieved": inst / (t_cap * 1e-3), "peak": issue_peak(clk),
                 "frac": inst / (t_cap * 1e-3) / issue_peak(clk),
                 "note": "the neighbour passes are bound by instruction issue, not HBM: instructions per launch "
                         "at this step (ncu, profiles/c2_dram_traffic.txt) over the live time per launch of the "
                         "same step; peak = 4 warp-instructions per cycle per SM x SMs x sampled SM clock"}

    line = {
        "metric": cfg.get("metric", METRIC), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded jittered lattice, mt19937_64 0xC0FFEE)",
        "config": config_record(cfg, n, nc, world, args),
        "e2e": {"value": e2e_units / e2e_total, "unit": UNIT, "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 32 * n,
                "steps": e2e_steps, "api": "pbf_step_host (pinned host pos/vel in, one step, pos/vel out)",
                "final_state_identical_to_timed_run": bool(e2e_steps == args.steps and
                                                           np.array_equal(e2e_pos, final_pos))},
        "roofline": {"bound": "hbm", "kernel": dom, "launches_per_step": len(members), "achieved": achieved,
                     "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "peak_kind": peak_kind, "traffic": traffic,
                     "traffic_step": cap_step,
                     "alg_bytes_per_launch": dom_bytes, "ms_per_launch": dom_ms,
                     "share_of_step": dom_step_ms / total_phase,
                     "window": "phase times averaged over the timed steps, replayed with events between phases"},
        "issue_roofline": issue,
        "step_roofline": {"alg_bytes_per_particle_step": step_alg_bytes(nc, cfg["iters"]),
                          "achieved": value * step_alg_bytes(nc, cfg["iters"]) / 1e9, "peak": hbm_peak,
                          "unit": "GB/s",
                          "frac": value * step_alg_bytes(nc, cfg["iters"]) / 1e9 / hbm_peak,
                          "dram_bytes_per_step": step_traffic, "dram_step": cap_step,
                          "dram_over_alg": None if step_traffic is None else
                          step_traffic / (step_alg_bytes(nc, cfg["iters"]) * n)},
        "phase_ms": {k: round(v, 5) for k, v in avg.items()},
        "phase_sum_ms": round(total_phase, 5),
        "profiled_window_identical_to_timed_run": bool(np.array_equal(prof_pos, final_pos)),
        "density_error": dens,
        "other_arithmetic": {
            "arithmetic": other, "value": n / (other_ms * 1e-3), "unit": UNIT, "ms_per_step": other_ms,
            "speedup_vs_line": (1e3 * total_s / args.steps) / other_ms,
            "final_positions_max_abs_diff_vs_line": float(np.max(np.abs(other_pos[:, :3].astype(np.float64) -
                                                                        final_pos[:, :3]))),
            "what": "the same window timed in the other arithmetic mode (pbf_set_math_mode); exact = bit-identical "
                    "to the reference kernels, fast = within 1e-5 relative per step (tests/test_gpu_fast_math.py); "
                    "over 20+ steps the two trajectories separate as the dynamics amplify rounding"},
        "step_ms": {"first": round(step_ms[0], 4), "median": round(statistics.median(step_ms), 4),
                    "max": round(max(step_ms), 4), "last": round(step_ms[-1], 4)},
        "gpu_launches": launches,
        "autotune": tuned,
        "clocks": clk,
        "neighbour_lists": {"capacity": list_cap, "longest": list_longest, "overflowed": list_overflowed},
    }

    # The reference's own CUDA kernels (compiled from its sources for sm_103a,
    # driven in its phase order by oracle/ref/ref_harness.cu, one CUDA graph
    # per step as sim::Simulator does) over the same step window.
    if rank == 0 and world == 1 and not args.no_reference_gpu:
        ref = pbfx.load_ref()
        if ref is not None:
            rpos, rvel = pos.copy(), np.zeros_like(pos)
            ms = C.c_double()
            rc = ref.ref_time_steps(pp, 1 if hashed else 0, pbfx.ptr(rpos), pbfx.ptr(rvel), n, args.warmup, args.steps,
                                    C.byref(ms))
            if rc == 0:
                same = bool(np.array_equal(final_pos, rpos) and np.array_equal(final_vel, rvel))
                line["reference_gpu"] = {
                    "value": n / (ms.value * 1e-3), "unit": UNIT, "ms_per_step": ms.value,
                    "what": "reference kernels (sim/*.cu) built for sm_103a, same steps, graph per step, "
                            "no L2 flush between steps", "speedup": value / (n / (ms.value * 1e-3)),
                    "final_state_identical_to_timed_run": same}
                line["parity"] = {
                    "timed_run_vs_reference_kernels": "bit-identical" if same else "DIFFERENT",
                    "what": "positions and velocities after the warm-up and timed steps of the fused step (value) "
                            "against the reference's own kernels run over the same steps from the same lattice"}
                # the same steps through this library's reference-layout phase launchers
                lms, lpos = launcher_path(lib, p, pos, hashed, args.warmup, args.steps)
                line["launcher_path"] = {
                    "value": n / (lms * 1e-3), "unit": UNIT, "ms_per_step": lms,
                    "what": "pbf_launch_* in the reference's phase order, one launch at a time, same steps, "
                            "no L2 flush between steps", "speedup_vs_reference_kernels": ms.value / lms,
                    "final_state_identical_to_reference_kernels": bool(np.array_equal(lpos, rpos))}

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        orc = pbfx.load_oracle()
        rate, steps, secs = cpu_rate(orc, p, hashed, snap_pos, snap_vel, args.cpu_budget, 1 << 30)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": orc.oracle_num_threads(), "kind": "port",
                                "sample": "oracle FP32 steps %d..%d of the same run (%d particles), %.1f s" % (
                                    args.warmup, args.warmup + steps - 1, n, secs)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_adjoint(args, cfg, world, rank, local):
    """C5: reverse-mode gradients (pbf_forward / pbf_backward) vs the forward."""
    import torch

    import __graft_entry__ as g
    import pbfx

    if rank == 0 or world == 1:
        g.build_library()
    barrier(world)
    torch.cuda.set_device(local)
    lib = pbfx.load()
    nx, ny, nz = cfg["lattice"]
    n = nx * ny * nz
    T, K, res = cfg["horizon"], cfg["every"], cfg["res"]
    S = cfg["scenes"]
    sims, starts, targets = [], [], []
    try:
        for sc in range(S):
            p = pbfx.dam_break_params(cfg["box"], cfg["iters"], n)
            pos = pbfx.seed_lattice(lib, nx, ny, nz, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC5000 + sc, p)
            rng = np.random.default_rng(0xC5000 + sc)
            vstar = np.zeros_like(pos)
            vstar[:, :3] = rng.uniform(-0.3, 0.3, (n, 3))
            target = torch.zeros(res ** 3, dtype=torch.float32, device="cuda")
            s = pbfx.Sim(lib, p, hashed=cfg["hashed"])
            sims.append(s)
            s.upload(pos, vstar)  # target: the density after a run from seeded velocities
            s.step(T)
            pbfx.check(lib.pbf_density_grid(s.h, res, C.c_void_p(target.data_ptr())))
            s.upload(pos, np.zeros_like(pos))
            s.step(1)  # graph capture outside the timing
            starts.append(pos)
            targets.append(target)

        def adjoint_run(batched, pbar=None):
            """Forward T steps and backward of the 32 scenes from their seeded
            lattices at rest; (forward s, backward s, losses, dL/dv0, dL/dc,
            final positions, dL/dx_T).  pbar: dL/dx_T to use instead of the
            loss's (which scatters with float atomics, so its bits vary run
            to run)."""
            for s, pos in zip(sims, starts):
                s.upload(pos, np.zeros_like(pos))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if batched:
                tapes = pbfx.forward_batch(lib, sims, T, K)
            else:
                tapes = []
                for s in sims:
                    t = C.c_void_p()
                    pbfx.check(lib.pbf_forward(s.h, T, K, C.byref(t)))
                    tapes.append(t)
            torch.cuda.synchronize()
            fwd = time.perf_counter() - t0
            try:
                finals = [s.download()[0] for s in sims]
                fresh = pbar is None
                if fresh:
                    pbar = [torch.zeros((n, 4), dtype=torch.float32, device="cuda") for _ in range(S)]
                vbar = [torch.zeros_like(x) for x in pbar]
                g0 = [torch.zeros_like(x) for x in pbar]
                losses = []
                for s, tg, pb in zip(sims, targets, pbar):
                    loss = C.c_double()
                    pbfx.check(lib.pbf_density_grid_loss(s.h, res, C.c_void_p(tg.data_ptr()), C.byref(loss),
                                                         C.c_void_p(pb.data_ptr()) if fresh else None))
                    losses.append(loss.value)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                if batched:
                    cb = pbfx.backward_batch(lib, tapes, [x.data_ptr() for x in pbar], [x.data_ptr() for x in vbar],
                                             None, [x.data_ptr() for x in g0])
                else:
                    cb = []
                    for t, pb, vb, g in zip(tapes, pbar, vbar, g0):
                        c = C.c_float()
                        pbfx.check(lib.pbf_backward(t, C.c_void_p(pb.data_ptr()), C.c_void_p(vb.data_ptr()), None,
                                                    C.c_void_p(g.data_ptr()), C.byref(c)))
                        cb.append(c.value)
                torch.cuda.synchronize()
                bwd = time.perf_counter() - t0
                return fwd, bwd, losses, [x[:, :3].cpu().numpy() for x in g0], cb, finals, pbar
            finally:
                for t in tapes:
                    lib.pbf_tape_destroy(t)

        fwd_s, bwd_s, losses, grads, cbar, finals, pbar = adjoint_run(True)
        sfwd_s, sbwd_s, _, sgrads, scbar, sfinals, _ = adjoint_run(False, pbar)
    finally:
        for s in sims:
            s.close()
    same_state = all(np.array_equal(a, b) for a, b in zip(finals, sfinals))
    same_bits = all(np.array_equal(a, b, equal_nan=True) for a, b in zip(grads, sgrads)) and all(
        a == b or (a != a and b != b) for a, b in zip(cbar, scbar))
    gnorm = [float(np.linalg.norm(g)) for g in grads]
    finite = [float(np.isfinite(g).mean()) for g in grads]
    # Gradient norm against the horizon, first scene: the reference's default
    # constants make the step chaotic (FP32 and FP64 runs separate ~10x per
    # step), so |dL/dv0| grows geometrically with the horizon.
    growth, growth_finite, ratio_by_h = {}, {}, {}
    p = pbfx.dam_break_params(cfg["box"], cfg["iters"], n)
    pos = pbfx.seed_lattice(lib, nx, ny, nz, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC5000, p)
    for H in (1, 2, 4, 8, 16, 32, T):
        with pbfx.Sim(lib, p, hashed=cfg["hashed"]) as s:
            tgt = torch.zeros(res ** 3, dtype=torch.float32, device="cuda")
            s.upload(pos, np.zeros_like(pos))
            s.step(1)  # graph capture outside the timing
            s.upload(pos, np.zeros_like(pos))
            torch.cuda.synchronize()
            tape = C.c_void_p()
            t0 = time.perf_counter()
            pbfx.check(lib.pbf_forward(s.h, H, min(K, H), C.byref(tape)))
            torch.cuda.synchronize()
            tf = time.perf_counter() - t0
            try:
                pbar = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
                vbar, g0 = torch.zeros_like(pbar), torch.zeros_like(pbar)
                loss, cb = C.c_double(), C.c_float()
                pbfx.check(lib.pbf_density_grid_loss(s.h, res, C.c_void_p(tgt.data_ptr()), C.byref(loss),
                                                     C.c_void_p(pbar.data_ptr())))
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                pbfx.check(lib.pbf_backward(tape, C.c_void_p(pbar.data_ptr()), C.c_void_p(vbar.data_ptr()), None,
                                            C.c_void_p(g0.data_ptr()), C.byref(cb)))
                torch.cuda.synchronize()
                tb = time.perf_counter() - t0
                growth[str(H)] = float(torch.linalg.norm(g0[:, :3]).item())
                growth_finite[str(H)] = float(torch.isfinite(g0[:, :3]).float().mean().item())
                ratio_by_h[str(H)] = tb / tf
            finally:
                lib.pbf_tape_destroy(tape)
    ratio = bwd_s / fwd_s
    line = {
        "metric": "adjoint/fwd time", "value": ratio, "unit": "backward time / forward time", "n_gpus": world,
        "steps": T, "warmup": 1, "ms_per_step": 1e3 * (fwd_s + bwd_s) / (S * T), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattices)",
        "config": {"workload": cfg["workload"], "scenes": S, "particles_per_scene": n, "solver_iters": cfg["iters"],
                   "checkpoint_every": K, "grid_points": res ** 3, "parallelism": "single"},
        "forward_ms_per_step": 1e3 * fwd_s / (S * T), "backward_ms_per_step": 1e3 * bwd_s / (S * T),
        "timed": "the 32 scenes as one batch: pbf_forward_batch (each scene's steps on its own stream, one "
                 "synchronisation) and pbf_backward_batch; per step = per scene-step of the batch",
        "backward_includes": "the replay of each checkpoint segment (one recorded forward step per step) and the "
                             "adjoint kernels",
        "scene_by_scene": {"value": sbwd_s / sfwd_s, "forward_ms_per_step": 1e3 * sfwd_s / (S * T),
                           "backward_ms_per_step": 1e3 * sbwd_s / (S * T),
                           "batch_speedup": (sfwd_s + sbwd_s) / (fwd_s + bwd_s),
                           "final_states_identical_to_batch": bool(same_state),
                           "gradients_identical_to_batch": bool(same_bits),
                           "what": "the same 32 scenes through pbf_forward / pbf_backward one scene at a time "
                                   "(each call synchronises), from the same states and with the batch's dL/dx_T"},
        "loss_mean": float(np.mean(losses)), "grad_v0_norm_mean": float(np.mean(gnorm)),
        "grad_xsph_c_mean": float(np.mean(cbar)),
        "grad_v0_norm_by_horizon": growth,
        "grad_v0_finite_fraction": float(np.mean(finite)),
        "grad_v0_finite_fraction_by_horizon": growth_finite,
        "backward_over_forward_by_horizon": ratio_by_h,
        "gradient_note": "the reference's default constants make the step chaotic (FP32 and FP64 runs separate "
                         "~10x per step), so |dL/dv0| grows geometrically with the horizon and overflows FP32 "
                         "before 60 steps; the time ratio is also reported per horizon, where the gradient is "
                         "finite (1-16 steps).  Per-step vector-Jacobian products are checked against an FP64 tape "
                         "in tests/test_gpu_adjoint_vjp.py",
        "e2e": {"value": ratio, "unit": "backward time / forward time", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0, "note": "host wall clock around pbf_forward_batch / pbf_backward_batch"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_ensemble(args, cfg, world, rank, local):
    """C4: the batched ensemble vs the same scenes stepped one by one."""
    import torch

    import __graft_entry__ as g
    import pbfx

    if rank == 0 or world == 1:
        g.build_library()
        g.build_oracle()
    barrier(world)
    torch.cuda.set_device(local)
    lib = pbfx.load()
    scenes, pos = pbfx.ensemble_scenes(lib, cfg["scenes"], seed=cfg["seed"])
    vel = np.zeros_like(pos)
    S, n = len(scenes), pos.shape[0]
    ens = pbfx.Ensemble(lib, scenes)
    ens.upload(pos, vel)
    stream = torch.cuda.ExternalStream(ens.stream_ptr())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    pbfx.check(lib.pbf_ensemble_step(ens.h, args.warmup))
    pbfx.check(lib.pbf_ensemble_synchronize(ens.h))
    tuned = None
    if args.autotune_steps > 0:  # untimed; the tuner puts the state back
        tuned = tuning_report(lib, *ens.autotune(steps=args.autotune_steps), args.autotune_steps,
                              "pbf_ensemble_autotune")
    snap_pos, snap_vel = ens.download()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler()
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()  # L2 flush, outside the timed window
            ev[k][0].record(stream)
            lib.pbf_ensemble_step(ens.h, 1)
            ev[k][1].record(stream)
    pbfx.check(lib.pbf_ensemble_synchronize(ens.h))
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop(None)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_s, units = aggregate(sum(step_ms) / 1e3, float(S) * args.steps, world)
    value = units / total_s

    dens = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        dens = ensemble_density_error(ens, scenes, pbfx.load_oracle())

    # End to end: host state in and out every step.
    hp = torch.from_numpy(snap_pos.copy()).pin_memory()
    hv = torch.from_numpy(snap_vel.copy()).pin_memory()
    e2e_steps = e2e_step_count(args)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        pbfx.check(lib.pbf_ensemble_step_host(ens.h, C.c_void_p(hp.data_ptr()), C.c_void_p(hv.data_ptr())))
    e2e_s = time.perf_counter() - t0
    launches = ens.launches_per_step() * args.steps
    ens.close()

    # Looped: every scene its own pbf_sim, stepped scene after scene from the
    # same post-warm-up state (each handle on its own stream, so neighbouring
    # scenes' launches may overlap on the GPU).
    loop_steps = args.steps if args.loop_steps <= 0 else max(1, min(args.steps, args.loop_steps))
    off = np.zeros(S + 1, np.int64)
    off[1:] = np.cumsum([p.numParticles for p in scenes])
    sims = []
    for k, p in enumerate(scenes):
        sm = pbfx.Sim(lib, p, hashed=True)
        sm.upload(snap_pos[off[k]:off[k + 1]], snap_vel[off[k]:off[k + 1]])
        sims.append(sm)
    for sm in sims:  # graph capture and upload, outside the timing
        pbfx.check(lib.pbf_step(sm.h, None))
    torch.cuda.synchronize()
    for k, sm in enumerate(sims):
        sm.upload(snap_pos[off[k]:off[k + 1]], snap_vel[off[k]:off[k + 1]])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(loop_steps):
        for sm in sims:
            lib.pbf_step(sm.h, None)
    for sm in sims:
        pbfx.check(lib.pbf_synchronize(sm.h))
    loop_s = time.perf_counter() - t0
    # Serial: one scene-step at a time, each completed before the next (a
    # single simulator stepping the scenes in turn).
    serial_steps = max(1, min(loop_steps, 5))
    for k, sm in enumerate(sims):
        sm.upload(snap_pos[off[k]:off[k + 1]], snap_vel[off[k]:off[k + 1]])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(serial_steps):
        for sm in sims:
            lib.pbf_step(sm.h, None)
            pbfx.check(lib.pbf_synchronize(sm.h))
    serial_s = time.perf_counter() - t0
    for sm in sims:
        sm.close()
    looped = S * loop_steps / loop_s
    looped_serial = S * serial_steps / serial_s

    line = {
        "metric": "scene-steps/s (ensemble of 256 scenes)", "value": value, "unit": "scene-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (pbfx.ensemble_scenes, seed 0x%X)" % cfg["seed"],
        "config": {"workload": cfg["workload"], "scenes": S, "particles": n,
                   "particles_per_scene": [int(min(p.numParticles for p in scenes)),
                                           int(max(p.numParticles for p in scenes))],
                   "parallelism": "replicas" if world > 1 else "single",
                   "timed_steps": "steps %d..%d of the run from the seeded lattices" % (
                       args.warmup, args.warmup + args.steps - 1),
                   "l2": "flushed before every timed step (256 MiB write, untimed)"},
        "particle_steps_per_s": n * args.steps / total_s,
        "looped": {"value": looped, "unit": "scene-steps/s", "steps": loop_steps,
                   "what": "each scene its own pbf_sim (fused step, one graph per scene-step, one stream per "
                           "scene so scenes overlap on the GPU), host loop over scenes, same post-warm-up state, "
                           "wall clock",
                   "speedup_of_ensemble": value / looped},
        "looped_serial": {"value": looped_serial, "unit": "scene-steps/s", "steps": serial_steps,
                          "what": "the same pbf_sims stepped one scene at a time, each step completed before the "
                                  "next, from the same state, wall clock",
                          "speedup_of_ensemble": value / looped_serial},
        "e2e": {"value": S * e2e_steps / e2e_s, "unit": "scene-steps/s", "h2d_bytes_per_step": 32 * n,
                "d2h_bytes_per_step": 32 * n, "steps": e2e_steps,
                "api": "pbf_ensemble_step_host (pinned host pos/vel in, one step, pos/vel out)"},
        "step_ms": {"first": round(step_ms[0], 4), "median": round(statistics.median(step_ms), 4),
                    "max": round(max(step_ms), 4), "last": round(step_ms[-1], 4)},
        "gpu_launches": launches,
        "autotune": tuned,
        "clocks": clk,
        "density_error": dens,
    }

    # The reference's own kernels looped scene by scene (graph per step).
    if rank == 0 and world == 1 and not args.no_reference_gpu:
        ref = pbfx.load_ref()
        if ref is not None:
            total_ms = 0.0
            ok = True
            for k, p in enumerate(scenes):
                rp = np.ascontiguousarray(snap_pos[off[k]:off[k + 1]])
                rv = np.ascontiguousarray(snap_vel[off[k]:off[k + 1]])
                ms = C.c_double()
                if ref.ref_time_steps(C.byref(p), 1, pbfx.ptr(rp), pbfx.ptr(rv), int(p.numParticles), 0,
                                      loop_steps, C.byref(ms)) != 0:
                    ok = False
                    break
                total_ms += ms.value * loop_steps
            if ok:
                line["reference_gpu_looped"] = {
                    "value": S * loop_steps / (total_ms * 1e-3), "unit": "scene-steps/s",
                    "what": "reference kernels (sim/*.cu) built for sm_103a, each scene stepped alone, device time "
                            "of its graphs summed over scenes (launch gaps between scenes not counted)",
                    "speedup_of_ensemble": value / (S * loop_steps / (total_ms * 1e-3))}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--autotune-steps", type=int, default=3,
                    help="steps per tile shape for the autotuner after warm-up (0: keep the default shape)")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--math", choices=["exact", "fast"], default="exact",
                    help="arithmetic of the lambda / delta passes: exact (bit-identical to the reference kernels) "
                         "or fast (within 1e-5 relative per step)")
    ap.add_argument("--config", choices=sorted(CONFIGS), default="c2")
    ap.add_argument("--profile-steps", type=int, default=5)
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="steps of the end-to-end measurement; 0 = the timed steps, the same window as value")
    ap.add_argument("--cpu-budget", type=float, default=10.0, help="seconds of CPU-baseline work")
    ap.add_argument("--ref-budget", type=float, default=150.0, help="seconds cap of the reference arm")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true")
    ap.add_argument("--loop-steps", type=int, default=0,
                    help="steps of the looped baseline (c4); 0 = the timed steps, the same window as the ensemble")
    ap.add_argument("--scenes", type=int, default=0,
                    help="number of scenes of c4 / c5 (0: the configuration's; fewer make small profiling runs)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    world, rank, local = dist_setup()
    cfg = CONFIGS[args.config]
    if args.scenes > 0 and "scenes" in cfg and args.scenes != cfg["scenes"]:
        cfg = dict(cfg, scenes=args.scenes)
        cfg["workload"] += " [run with %d scenes]" % args.scenes
    if args.impl == "reference":
        if cfg.get("adjoint"):
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no adjoint"}))
            return 0
        if "scenes" in cfg:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched ensemble; "
                              "bench.py --config c4 reports its looped kernels as reference_gpu_looped"}))
            return 0
        return run_reference(args, cfg, world, rank)
    if cfg.get("adjoint"):
        return run_adjoint(args, cfg, world, rank, local)
    if "scenes" in cfg:
        return run_ensemble(args, cfg, world, rank, local)
    return run_ours(args, cfg, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
