"""C-ABI checks that need no GPU: exports, struct layout, parameter helpers."""
import ctypes as C
import os
import re

import numpy as np

import pbfx

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "pbf", h) for h in ("pbf.h", "launch_abi.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(?:int|void|bool|const char\*|void\*)\s+\**\s*((?:pbf_|Launch|Ensure)\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 40, names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_launcher_names_exported(lib):
    for n in ("LaunchIntegratePred", "LaunchBoundary", "LaunchVelocity", "LaunchHashKeys", "LaunchSortPairsQuery",
              "LaunchSortPairs", "LaunchCellRanges", "LaunchCellRangesCompact", "EnsureCellCompactScratch",
              "LaunchLambda", "LaunchLambdaCompact", "LaunchDeltaApply", "LaunchDeltaApplyCompact", "LaunchXSPH",
              "LaunchXSPHCompact"):
        assert hasattr(lib, n), n


def test_struct_sizes_match_library(lib):
    sz = (C.c_uint32 * 5)()
    lib.pbf_abi_sizes(C.byref(sz))
    assert list(sz) == [C.sizeof(t) for t in (pbfx.KernelCoeffs, pbfx.GridBounds, pbfx.Tuning, pbfx.SimParams,
                                              pbfx.DeviceParams)]
    # reference sim/parameters.h layout: 6 + 10 + 22 floats/ints
    assert list(sz)[:3] == [24, 40, 88]


def test_default_tuning_matches_reference(lib):
    t = pbfx.Tuning()
    lib.pbf_default_tuning(C.byref(t))
    # sim/parameters.h:27-57
    assert (t.scorr_enable, t.xpbd_enable, t.enable_lambda_clamp, t.enable_disp_clamp, t.enable_relax) == (1, 0, 1, 1, 1)
    np.testing.assert_array_equal(
        np.float32([t.scorr_k, t.scorr_n, t.scorr_dq_h, t.wq_min, t.scorr_min, t.grad_r_eps, t.lambda_denom_eps,
                    t.lambda_max_abs, t.disp_clamp_max_h, t.relax_omega]),
        np.float32([0.003, 4.0, 0.3, 1e-12, -0.25, 1e-6, 1e-4, 50.0, 0.05, 0.75]))
    assert (t.xsph_n_min, t.xsph_n_max) == (0, 8)


def test_kernel_coeffs_fp32(lib):
    kc = pbfx.KernelCoeffs()
    h = np.float32(2.5) * np.float32(0.005)
    lib.pbf_make_kernel_coeffs(float(h), C.byref(kc))
    # sim/parameters.h:94-107 evaluated in FP32 in the same order
    f = np.float32
    pi = f(3.14159265358979323846)
    h2 = f(h * h)
    h3 = f(h * h2)
    h6 = f(h3 * h3)
    h9 = f(h6 * h3)
    assert kc.h == h and kc.h2 == h2
    assert f(kc.poly6) == f(f(315.0) / f(f(f(64.0) * pi) * h9))
    assert f(kc.spiky) == f(f(15.0) / f(pi * h6))


def test_grid_dims_fp32_rounding(lib):
    # h = 2.5f * 0.005f = 0.012499999f, so ceil(1/h) = 81, ceil(2/h) = 161,
    # ceil(3/h) = 241 (GridSystem::ComputeDims, sim/grid_system.h:9-17).
    for box, dims in (((1, 1, 1), (81, 81, 81)), ((2, 1, 2), (161, 81, 161)), ((3, 2, 3), (241, 161, 241))):
        p = pbfx.dam_break_params(box, 2, 10)
        assert (p.grid.dim.x, p.grid.dim.y, p.grid.dim.z) == dims
        d = (C.c_int32 * 3)()
        lib.pbf_compute_dims(C.byref(p.grid), C.byref(d))
        assert tuple(d) == dims


def test_dam_break_constants(lib):
    p = pbfx.dam_break_params((2, 1, 2), 2, 1 << 20)
    f = np.float32
    assert p.dt == f(1.0) / f(120.0)
    assert (p.gravity.x, p.gravity.y, p.gravity.z) == (0.0, f(-9.8), 0.0)
    assert p.solverIters == 2 and p.maxNeighbors == 64
    assert p.pbf.lambda_denom_eps == 100.0 and p.pbf.scorr_k == f(0.1) and p.pbf.scorr_dq_h == f(0.2)
    assert p.pbf.compliance == 0.0 and p.xsph_c == f(0.01) and p.boundaryRestitution == 0.0
    assert p.grid.cellSize == p.kernel.h
    # rest density = 6 face neighbours of the unjittered lattice
    hr2 = f(p.kernel.h2 - f(f(0.01) * f(0.01)))
    w = f(f(f(f(p.particleMass) * f(p.kernel.poly6)) * hr2) * hr2) * hr2
    acc = f(0)
    for _ in range(6):
        acc = f(acc + w)
    assert p.restDensity == acc
    assert abs(p.restDensity - 6 * 1e-3 * 37424.68) < 0.05


def test_seed_lattice_deterministic(lib):
    p = pbfx.dam_break_params((1, 1, 1), 2, 4 ** 3)
    a = pbfx.seed_lattice(lib, 4, 4, 4, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    b = pbfx.seed_lattice(lib, 4, 4, 4, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    assert np.array_equal(a, b)
    base = np.stack(np.meshgrid(np.arange(4), np.arange(4), np.arange(4), indexing="ij"), -1)[..., ::-1]
    base = (0.005 + base.reshape(-1, 3) * 0.01)
    assert np.all(np.abs(a[:, :3] - base) <= 0.0005 + 1e-7)
    assert np.all(a[:, 3] == 1.0)
    c = pbfx.seed_lattice(lib, 4, 4, 4, (0.005, 0.005, 0.005), 0.01, 0.0005, 1234, p)
    assert not np.array_equal(a, c)


def test_invalid_arguments_rejected_without_gpu(lib):
    assert lib.pbf_dam_break_params(-1.0, 1.0, 1.0, 2, 10, None) == pbfx.PBF_ERR_INVALID
    assert lib.pbf_launch_hash_keys(None, None, None, None, 5, None) == pbfx.PBF_ERR_INVALID
    assert lib.pbf_launch_sort_pairs(None, 0, None, None, None, None, 5, None) == pbfx.PBF_ERR_INVALID
    # N == 0 is a no-op success (reference launchers return early)
    assert lib.pbf_launch_hash_keys(None, None, None, None, 0, None) == pbfx.PBF_OK
    out = C.c_size_t()
    assert lib.pbf_sort_pairs_query(C.byref(out), 1000) == pbfx.PBF_OK and out.value > 8000
    assert lib.pbf_status_string(pbfx.PBF_ERR_TIMEOUT) == b"bounded device wait gave up"
