"""Pins the CPU oracle against known answers (no GPU).

* tests/golden/kat_formulas.json: FP64 restatement of the reference formulas
  (generated by tests/golden/make_kat.py, independent of the oracle code).
* Integer phases (keys, stable sort, dense and compact cell tables) against
  numpy restatements, bit-exact, including edge cases.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

import pbfx

HERE = os.path.dirname(os.path.abspath(__file__))
KAT = json.load(open(os.path.join(HERE, "golden", "kat_formulas.json")))

# FP32 oracle vs FP64 formulas: |a - b| <= TOL * max(|b|, floor), floor = 1%
# of the largest |b| of the quantity; normwise (floor = largest |b|) for the
# position correction, a sum of cancelling neighbour terms whose exact value
# can be 0 while FP32 leaves ~1e-6 of the summands.
TOL = 1e-5


def kat_params(lib, c):
    prm = c["params"]
    p = pbfx.dam_break_params((1.0, 1.0, 1.0), 1, len(c["pos"]))
    lib.pbf_make_kernel_coeffs(prm["h"], C.byref(p.kernel))
    p.grid.cellSize = prm["cell_size"]
    p.grid.dim.x, p.grid.dim.y, p.grid.dim.z = prm["dim"]
    p.particleMass = prm["mass"]
    p.restDensity = prm["rest_density"]
    p.pbf.lambda_denom_eps = prm["lambda_denom_eps"]
    p.pbf.lambda_max_abs = prm["lambda_max_abs"]
    p.maxNeighbors = prm["max_neighbors"]
    p.xsph_c = prm["xsph_c"]
    return p


def f4(rows, w):
    a = np.zeros((len(rows), 4), np.float32)
    a[:, :3] = np.float32(rows)
    a[:, 3] = w
    return a


def build_grid(orc, p, pred, hashed):
    n = pred.shape[0]
    keys = np.zeros(n, np.uint32)
    idx = np.zeros(n, np.uint32)
    orc.oracle_hash_keys(pbfx.ptr(keys), pbfx.ptr(idx), pbfx.ptr(pred), C.byref(p.grid), n)
    ks = np.zeros(n, np.uint32)
    is_ = np.zeros(n, np.uint32)
    orc.oracle_sort_pairs(pbfx.ptr(keys), pbfx.ptr(ks), pbfx.ptr(idx), pbfx.ptr(is_), n)
    t = pbfx.OracleTable()
    keep = [keys, ks, is_]
    if hashed:
        uk = np.zeros(max(n, 1), np.uint32)
        off = np.zeros(n + 1, np.uint32)
        cnt = np.zeros(1, np.uint32)
        orc.oracle_cell_ranges_compact(pbfx.ptr(uk), pbfx.ptr(off), pbfx.ptr(cnt), pbfx.ptr(ks), n)
        t.unique_keys, t.offsets, t.count = uk.ctypes.data, off.ctypes.data, int(cnt[0])
        keep += [uk, off, cnt]
    else:
        nc = pbfx.num_cells(p)
        st = np.zeros(nc, np.uint32)
        en = np.zeros(nc, np.uint32)
        orc.oracle_cell_ranges(pbfx.ptr(st), pbfx.ptr(en), pbfx.ptr(ks), n, nc)
        t.start, t.end = st.ctypes.data, en.ctypes.data
        keep += [st, en]
    return keys, ks, is_, t, keep


@pytest.mark.parametrize("hashed", [False, True])
@pytest.mark.parametrize("case", KAT, ids=[c["name"] for c in KAT])
def test_oracle_matches_formulas(lib, orc, case, hashed):
    p = kat_params(lib, case)
    dp = pbfx.device_params(p)
    n = len(case["pos"])
    pred = f4(case["pos"], 1.0)
    keys, ks, is_, t, keep = build_grid(orc, p, pred, hashed)
    assert keys.tolist() == case["keys"]
    assert is_.tolist() == case["sorted_ids"]
    lam = np.zeros(n, np.float32)
    orc.oracle_lambda(pbfx.ptr(lam), pbfx.ptr(pred), pbfx.ptr(is_), pbfx.ptr(ks), C.byref(t), C.byref(dp), n)
    pbfx.assert_close(lam, case["lambda"], TOL, "lambda")
    # delta uses the KAT lambdas (as the reference's Jacobi pass would)
    lam64 = np.float32(case["lambda"])
    pred2 = pred.copy()
    delta = np.zeros_like(pred)
    orc.oracle_delta_apply(pbfx.ptr(pred2), pbfx.ptr(delta), pbfx.ptr(lam64), pbfx.ptr(is_), pbfx.ptr(ks), C.byref(t),
                           C.byref(dp), n)
    pbfx.assert_close(delta[:, :3], case["delta"], TOL, "delta", floor_frac=1.0)
    assert np.all(delta[:, 3] == 0.0)
    np.testing.assert_array_equal(pred2[:, :3], pred[:, :3] + delta[:, :3])
    vel = f4(case["vel"], 0.0)
    vout = np.zeros_like(vel)
    orc.oracle_xsph(pbfx.ptr(vout), pbfx.ptr(vel), pbfx.ptr(pred), pbfx.ptr(is_), pbfx.ptr(ks), C.byref(t),
                    C.byref(dp), n)
    pbfx.assert_close(vout[:, :3], case["xsph_vel"], TOL, "xsph")


def np_keys(pred, p):
    f = np.float32
    cs = f(p.grid.cellSize)
    mins = np.float32([p.grid.mins.x, p.grid.mins.y, p.grid.mins.z])
    dims = np.int64([p.grid.dim.x, p.grid.dim.y, p.grid.dim.z])
    rel = (pred[:, :3] - mins) / cs  # IEEE float32 divide
    c = np.floor(rel).astype(np.int64)
    c = np.clip(c, 0, dims - 1)
    return ((c[:, 2] * dims[1] + c[:, 1]) * dims[0] + c[:, 0]).astype(np.uint32)


def test_hash_keys_bit_exact_at_cell_boundaries(lib, orc):
    p = pbfx.dam_break_params((2.0, 1.0, 2.0), 2, 0)
    f = np.float32
    h = f(p.grid.cellSize)
    k = np.arange(0, 161, dtype=np.float32)
    edges = np.concatenate([k * h, np.nextafter(k * h, f(-1)), np.nextafter(k * h, f(3)), [f(-0.5), f(2.0), f(7.0)]])
    rng = np.random.default_rng(5)
    pts = np.stack([rng.choice(edges, 4096), rng.choice(np.clip(edges, 0, 1.2), 4096), rng.choice(edges, 4096)], 1)
    pred = np.zeros((4096, 4), np.float32)
    pred[:, :3] = pts
    keys = np.zeros(4096, np.uint32)
    idx = np.zeros(4096, np.uint32)
    orc.oracle_hash_keys(pbfx.ptr(keys), pbfx.ptr(idx), pbfx.ptr(pred), C.byref(p.grid), 4096)
    np.testing.assert_array_equal(keys, np_keys(pred, p))
    np.testing.assert_array_equal(idx, np.arange(4096, dtype=np.uint32))


@pytest.mark.parametrize("n,hi", [(0, 10), (1, 10), (2, 2), (1000, 3), (5000, 1 << 32), (4096, 1)])
def test_sort_pairs_stable(orc, n, hi):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    vals = rng.permutation(n).astype(np.uint32)
    ko = np.zeros(n, np.uint32)
    vo = np.zeros(n, np.uint32)
    orc.oracle_sort_pairs(pbfx.ptr(keys), pbfx.ptr(ko), pbfx.ptr(vals), pbfx.ptr(vo), n)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(ko, keys[order])
    np.testing.assert_array_equal(vo, vals[order])


def np_dense(ks, n, nc):
    st = np.full(nc, 0xFFFFFFFF, np.uint32)
    en = np.zeros(nc, np.uint32)
    if n:
        u, first, cnt = np.unique(ks, return_index=True, return_counts=True)
        ok = u < nc
        st[u[ok]] = first[ok]
        en[u[ok]] = (first + cnt)[ok]
    return st, en


@pytest.mark.parametrize("n", [0, 1, 7, 3000])
def test_cell_tables(orc, n):
    rng = np.random.default_rng(n + 1)
    nc = 500
    ks = np.sort(rng.integers(0, nc, n).astype(np.uint32))
    st = np.zeros(nc, np.uint32)
    en = np.zeros(nc, np.uint32)
    orc.oracle_cell_ranges(pbfx.ptr(st), pbfx.ptr(en), pbfx.ptr(ks), n, nc)
    est, een = np_dense(ks, n, nc)
    np.testing.assert_array_equal(st, est)
    np.testing.assert_array_equal(en, een)
    uk = np.zeros(max(n, 1), np.uint32)
    off = np.zeros(n + 1, np.uint32)
    cnt = np.zeros(1, np.uint32)
    orc.oracle_cell_ranges_compact(pbfx.ptr(uk), pbfx.ptr(off), pbfx.ptr(cnt), pbfx.ptr(ks), n)
    u, first = np.unique(ks, return_index=True)
    assert int(cnt[0]) == len(u)
    np.testing.assert_array_equal(uk[: len(u)], u)
    np.testing.assert_array_equal(off[: len(u)], first)
    assert off[len(u)] == n


def test_boundary_and_velocity(orc):
    p = pbfx.dam_break_params((1.0, 1.0, 1.0), 1, 4)
    pred = np.float32([[-0.5, 0.5, 1.5, 7.0], [0.2, -0.1, 0.3, 2.0], [0.5, 0.5, 0.5, 0.0], [2.0, 2.0, -3.0, 1.0]])
    vel = np.float32([[1.0, 2.0, 3.0, 9.0], [1.0, -2.0, 3.0, 9.0], [1.0, 2.0, 3.0, 9.0], [4.0, 5.0, -6.0, 9.0]])
    pr, ve = pred.copy(), vel.copy()
    orc.oracle_boundary(pbfx.ptr(pr), pbfx.ptr(ve), C.byref(p.grid), 0.5, 4)
    np.testing.assert_array_equal(pr, np.float32([[0, 0.5, 1, 1], [0.2, 0, 0.3, 1], [0.5, 0.5, 0.5, 1],
                                                  [1, 1, 0, 1]]))
    np.testing.assert_array_equal(ve, np.float32([[-0.5, 2, -1.5, 0], [1, 1, 3, 0], [1, 2, 3, 0], [-2, -2.5, 3, 0]]))
    # e = 0 keeps signed zeros: -0.0 * v
    pr, ve = pred.copy(), vel.copy()
    orc.oracle_boundary(pbfx.ptr(pr), pbfx.ptr(ve), C.byref(p.grid), 0.0, 4)
    assert np.signbit(ve[0, 0]) and ve[0, 0] == 0.0
    v2 = np.zeros_like(vel)
    orc.oracle_velocity(pbfx.ptr(v2), pbfx.ptr(pred), pbfx.ptr(pr), np.float32(120.0), 4)
    np.testing.assert_array_equal(v2[:, :3], (pr[:, :3] - pred[:, :3]) * np.float32(120.0))
    assert np.all(v2[:, 3] == 0)


def test_integrate_uses_fused_multiply_add(orc):
    # pred = fma(fma(g, dt, v), dt, p) per axis (the GPU's fused form).
    p = np.float32([[0.1, 0.2, 0.3, 5.0]])
    v = np.float32([[0.7, -0.3, 0.11, 0.0]])
    g = pbfx.Float3(0.0, np.float32(-9.8), 0.0)
    dt = np.float32(1.0) / np.float32(120.0)
    out = np.zeros_like(p)
    orc.oracle_integrate_pred(pbfx.ptr(p), pbfx.ptr(v), pbfx.ptr(out), g, dt, 1)

    def fma(a, b, c):
        return np.float32(np.float64(a) * np.float64(b) + np.float64(c))  # exact product, one rounding

    gv = [0.0, np.float32(-9.8), 0.0]
    exp = [fma(fma(gv[a], dt, v[0, a]), dt, p[0, a]) for a in range(3)]
    np.testing.assert_array_equal(out[0, :3], np.float32(exp))
    assert out[0, 3] == 5.0
