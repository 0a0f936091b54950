"""Phase launchers on the GPU vs the CPU oracle, through the C ABI.

Integer phases (hash keys, sort, dense and compact cell tables), lambda and
XSPH must be bit-exact; the position correction agrees within
parity.PHASE_DELTA (normwise; the oracle's powf is the C library's).  Inputs: seeded scenes of the dam-break configuration at
the lattice start and after the fluid has compressed (many neighbours, the
neighbour cap engaged), plus ragged and edge-case sizes.
"""
import ctypes as C

import numpy as np
import pytest

import pbfx
from parity import PHASE_DELTA, STEP_POS

pytestmark = pytest.mark.gpu


def D(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def P(t):
    return C.c_void_p(t.data_ptr())


def H(t):
    return t.cpu().numpy()


def sync(torch):
    torch.cuda.synchronize()


@pytest.fixture(scope="module")
def scenes(lib, orc):
    """(params, positions) pairs: C1 lattice start and a compressed state."""
    out = {}
    p = pbfx.dam_break_params((1.0, 1.0, 1.0), 2, 32 ** 3)
    pos = pbfx.seed_lattice(lib, 32, 32, 32, (0.005, 0.005, 0.005), 0.01, 0.0005, 0xC0FFEE, p)
    vel = np.zeros_like(pos)
    out["lattice"] = (p, pos.copy(), vel.copy())
    for _ in range(35):
        pbfx.oracle_step(orc, p, True, pos, vel, trace=False)
    out["compressed"] = (p, pos.copy(), vel.copy())
    return out


# ----------------------------------------------------------------- sort
SORT_CASES = [
    (1, "random"), (2, "random"), (31, "dup"), (2047, "random"), (2048, "dup"), (2049, "random"),
    (3839, "random"), (3840, "dup"), (3841, "random"), (7679, "random"), (7680, "dup"), (7681, "random"),
    (15_361, "random"), (524_287, "random"), (524_288, "dup"), (614_401, "random"),
    (100_000, "random"), (100_000, "dup"), (100_000, "equal"), (100_000, "sorted"), (100_000, "reverse"),
    (1 << 20, "cells"), (777_777, "random"),
]


def make_keys(n, kind, rng):
    if kind == "random":
        return rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    if kind == "dup":
        return rng.integers(0, 7, n).astype(np.uint32) * np.uint32(0x01010101)
    if kind == "equal":
        return np.full(n, 0xDEADBEEF, np.uint32)
    if kind == "sorted":
        return np.sort(rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32))
    if kind == "reverse":
        return np.sort(rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32))[::-1].copy()
    if kind == "cells":
        return rng.integers(0, 161 * 81 * 161, n).astype(np.uint32)
    raise ValueError(kind)


@pytest.mark.parametrize("n,kind", SORT_CASES)
def test_sort_pairs_bit_exact(gpu, lib, n, kind):
    torch = gpu
    rng = np.random.default_rng(n + len(kind))
    keys = make_keys(n, kind, rng)
    vals = rng.permutation(n).astype(np.uint32)
    order = np.argsort(keys, kind="stable")
    tb = C.c_size_t()
    pbfx.check(lib.pbf_sort_pairs_query(C.byref(tb), n))
    tmp = torch.empty(tb.value, dtype=torch.uint8, device="cuda")
    kin, vin = D(torch, keys.view(np.int32)), D(torch, vals.view(np.int32))
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    pbfx.check(lib.pbf_launch_sort_pairs(P(tmp), tb.value, P(kin), P(kout), P(vin), P(vout), n, None))
    sync(torch)
    np.testing.assert_array_equal(H(kout).view(np.uint32), keys[order])
    np.testing.assert_array_equal(H(vout).view(np.uint32), vals[order])
    np.testing.assert_array_equal(H(kin).view(np.uint32), keys)  # input intact
    # reference-name entry point, same result
    kout2, vout2 = torch.empty_like(kin), torch.empty_like(vin)
    lib.LaunchSortPairs(P(tmp), C.c_size_t(tb.value), P(kin), P(kout2), P(vin), P(vout2), C.c_uint32(n), None)
    sync(torch)
    assert torch.equal(kout, kout2) and torch.equal(vout, vout2)


def test_sort_pairs_bits_subset(gpu, lib):
    torch = gpu
    n = 300_000
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 1 << 22, n).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    tb = C.c_size_t()
    pbfx.check(lib.pbf_sort_pairs_query(C.byref(tb), n))
    tmp = torch.empty(tb.value, dtype=torch.uint8, device="cuda")
    kin, vin = D(torch, keys.view(np.int32)), D(torch, vals.view(np.int32))
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    pbfx.check(lib.pbf_launch_sort_pairs_bits(P(tmp), tb.value, P(kin), P(kout), P(vin), P(vout), n, 22, None))
    sync(torch)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(H(kout).view(np.uint32), keys[order])
    np.testing.assert_array_equal(H(vout).view(np.uint32), vals[order])


def test_sort_rejects_aliasing(gpu, lib):
    torch = gpu
    k = torch.zeros(10, dtype=torch.int32, device="cuda")
    tmp = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    assert lib.pbf_launch_sort_pairs(P(tmp), 1 << 20, P(k), P(k), P(k), P(k.clone()), 10, None) == pbfx.PBF_ERR_INVALID


# ------------------------------------------------------- keys and tables
@pytest.mark.parametrize("scene", ["lattice", "compressed"])
def test_hash_keys_and_tables_bit_exact(gpu, lib, orc, scenes, scene):
    torch = gpu
    p, pos, vel = scenes[scene]
    n = pos.shape[0]
    nc = pbfx.num_cells(p)
    dpos = D(torch, pos)
    keys = torch.empty(n, dtype=torch.int32, device="cuda")
    idx = torch.empty_like(keys)
    pbfx.check(lib.pbf_launch_hash_keys(P(keys), P(idx), P(dpos), C.byref(p.grid), n, None))
    sync(torch)
    ok = np.zeros(n, np.uint32)
    oi = np.zeros(n, np.uint32)
    orc.oracle_hash_keys(pbfx.ptr(ok), pbfx.ptr(oi), pbfx.ptr(pos), C.byref(p.grid), n)
    np.testing.assert_array_equal(H(keys).view(np.uint32), ok)
    np.testing.assert_array_equal(H(idx).view(np.uint32), oi)
    ks = np.zeros(n, np.uint32)
    is_ = np.zeros(n, np.uint32)
    orc.oracle_sort_pairs(pbfx.ptr(ok), pbfx.ptr(ks), pbfx.ptr(oi), pbfx.ptr(is_), n)
    dks = D(torch, ks.view(np.int32))
    st = torch.empty(nc, dtype=torch.int32, device="cuda")
    en = torch.empty_like(st)
    pbfx.check(lib.pbf_launch_cell_ranges(P(st), P(en), P(dks), n, nc, None))
    ost, oen = np.zeros(nc, np.uint32), np.zeros(nc, np.uint32)
    orc.oracle_cell_ranges(pbfx.ptr(ost), pbfx.ptr(oen), pbfx.ptr(ks), n, nc)
    sync(torch)
    np.testing.assert_array_equal(H(st).view(np.uint32), ost)
    np.testing.assert_array_equal(H(en).view(np.uint32), oen)
    sb = C.c_size_t()
    pbfx.check(lib.pbf_cell_compact_scratch_query(C.byref(sb), n))
    scratch = torch.empty(sb.value, dtype=torch.uint8, device="cuda")
    uk = torch.empty(n, dtype=torch.int32, device="cuda")
    off = torch.empty(n + 1, dtype=torch.int32, device="cuda")
    cnt = torch.empty(1, dtype=torch.int32, device="cuda")
    pbfx.check(lib.pbf_launch_cell_ranges_compact(P(scratch), sb.value, P(uk), P(off), P(cnt), P(dks), n, None))
    ouk, ooff, ocnt = np.zeros(n, np.uint32), np.zeros(n + 1, np.uint32), np.zeros(1, np.uint32)
    orc.oracle_cell_ranges_compact(pbfx.ptr(ouk), pbfx.ptr(ooff), pbfx.ptr(ocnt), pbfx.ptr(ks), n)
    sync(torch)
    m = int(ocnt[0])
    assert int(H(cnt)[0]) == m
    np.testing.assert_array_equal(H(uk).view(np.uint32)[:m], ouk[:m])
    np.testing.assert_array_equal(H(off).view(np.uint32)[: m + 1], ooff[: m + 1])


@pytest.mark.parametrize("n", [0, 1, 2, 33, 2047, 2048, 2049, 4095, 4096, 4097, 70_001])
def test_compact_and_dense_ragged(gpu, lib, orc, n):
    torch = gpu
    rng = np.random.default_rng(n + 11)
    nc = 4000
    ks = np.sort(rng.integers(0, nc, n).astype(np.uint32))
    dks = D(torch, ks.view(np.int32)) if n else torch.empty(1, dtype=torch.int32, device="cuda")
    sb = C.c_size_t()
    pbfx.check(lib.pbf_cell_compact_scratch_query(C.byref(sb), max(n, 1)))
    scratch = torch.empty(sb.value, dtype=torch.uint8, device="cuda")
    uk = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    off = torch.full((n + 1,), -7, dtype=torch.int32, device="cuda")
    cnt = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    pbfx.check(lib.pbf_launch_cell_ranges_compact(P(scratch), sb.value, P(uk), P(off), P(cnt), P(dks), n, None))
    sync(torch)
    u, first = np.unique(ks, return_index=True)
    assert int(H(cnt)[0]) == len(u)
    np.testing.assert_array_equal(H(uk).view(np.uint32)[: len(u)], u)
    np.testing.assert_array_equal(H(off).view(np.uint32)[: len(u)], first)
    assert int(H(off)[len(u)]) == n
    st = torch.empty(nc, dtype=torch.int32, device="cuda")
    en = torch.empty_like(st)
    pbfx.check(lib.pbf_launch_cell_ranges(P(st), P(en), P(dks), n, nc, None))
    ost, oen = np.zeros(nc, np.uint32), np.zeros(nc, np.uint32)
    orc.oracle_cell_ranges(pbfx.ptr(ost), pbfx.ptr(oen), pbfx.ptr(ks), n, nc)
    sync(torch)
    np.testing.assert_array_equal(H(st).view(np.uint32), ost)
    np.testing.assert_array_equal(H(en).view(np.uint32), oen)


# ------------------------------------------------------- neighbour phases
def grid_inputs(orc, p, pred, hashed):
    n = pred.shape[0]
    keys, idx = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
    orc.oracle_hash_keys(pbfx.ptr(keys), pbfx.ptr(idx), pbfx.ptr(pred), C.byref(p.grid), n)
    ks, is_ = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
    orc.oracle_sort_pairs(pbfx.ptr(keys), pbfx.ptr(ks), pbfx.ptr(idx), pbfx.ptr(is_), n)
    t = pbfx.OracleTable()
    arrays = {"ks": ks, "is": is_}
    if hashed:
        uk, off, cnt = np.zeros(n, np.uint32), np.zeros(n + 1, np.uint32), np.zeros(1, np.uint32)
        orc.oracle_cell_ranges_compact(pbfx.ptr(uk), pbfx.ptr(off), pbfx.ptr(cnt), pbfx.ptr(ks), n)
        t.unique_keys, t.offsets, t.count = uk.ctypes.data, off.ctypes.data, int(cnt[0])
        arrays.update(uk=uk, off=off, cnt=cnt)
    else:
        nc = pbfx.num_cells(p)
        st, en = np.zeros(nc, np.uint32), np.zeros(nc, np.uint32)
        orc.oracle_cell_ranges(pbfx.ptr(st), pbfx.ptr(en), pbfx.ptr(ks), n, nc)
        t.start, t.end = st.ctypes.data, en.ctypes.data
        arrays.update(st=st, en=en)
    return t, arrays


@pytest.mark.parametrize("hashed", [False, True])
@pytest.mark.parametrize("scene", ["lattice", "compressed"])
def test_lambda_delta_xsph_vs_oracle(gpu, lib, orc, scenes, scene, hashed):
    torch = gpu
    p, pos, vel0 = scenes[scene]
    n = pos.shape[0]
    dp = pbfx.device_params(p)
    # prediction as the step computes it (predict + boundary e=0)
    pred = np.zeros_like(pos)
    orc.oracle_integrate_pred(pbfx.ptr(pos), pbfx.ptr(vel0), pbfx.ptr(pred), p.gravity, p.dt, n)
    vtmp = vel0.copy()
    orc.oracle_boundary(pbfx.ptr(pred), pbfx.ptr(vtmp), C.byref(p.grid), 0.0, n)
    t, a = grid_inputs(orc, p, pred, hashed)
    dg = {k: D(torch, v.view(np.int32)) for k, v in a.items()}
    if hashed:
        tab = (P(dg["uk"]), P(dg["off"]), P(dg["cnt"]))
        lam_fn, del_fn, xs_fn = lib.pbf_launch_lambda_compact, lib.pbf_launch_delta_apply_compact, lib.pbf_launch_xsph_compact
    else:
        tab = (P(dg["st"]), P(dg["en"]))
        lam_fn, del_fn, xs_fn = lib.pbf_launch_lambda, lib.pbf_launch_delta_apply, lib.pbf_launch_xsph
    # lambda
    dpred = D(torch, pred)
    dlam = torch.empty(n, dtype=torch.float32, device="cuda")
    pbfx.check(lam_fn(P(dlam), P(dpred), P(dg["is"]), P(dg["ks"]), *tab, C.byref(dp), n, None))
    olam = np.zeros(n, np.float32)
    orc.oracle_lambda(pbfx.ptr(olam), pbfx.ptr(pred), pbfx.ptr(a["is"]), pbfx.ptr(a["ks"]), C.byref(t), C.byref(dp), n)
    sync(torch)
    np.testing.assert_array_equal(H(dlam), olam)
    # delta + apply on the same lambdas
    lam_in = D(torch, olam)
    dpred2 = D(torch, pred)
    ddelta = torch.empty_like(dpred2)
    pbfx.check(del_fn(P(dpred2), P(ddelta), P(lam_in), P(dg["is"]), P(dg["ks"]), *tab, C.byref(dp), n, None))
    opred2, odelta = pred.copy(), np.zeros_like(pred)
    orc.oracle_delta_apply(pbfx.ptr(opred2), pbfx.ptr(odelta), pbfx.ptr(olam), pbfx.ptr(a["is"]), pbfx.ptr(a["ks"]),
                           C.byref(t), C.byref(dp), n)
    sync(torch)
    pbfx.assert_close(H(ddelta)[:, :3], odelta[:, :3], PHASE_DELTA, "delta", floor_frac=1.0)
    pbfx.assert_close(H(dpred2), opred2, STEP_POS, "pred after apply")
    # XSPH, Jacobi
    vin = np.random.default_rng(1).normal(size=(n, 4)).astype(np.float32)
    dvin = D(torch, vin)
    dvout = torch.empty_like(dvin)
    pbfx.check(xs_fn(P(dvout), P(dvin), P(dpred), P(dg["is"]), P(dg["ks"]), *tab, C.byref(dp), n, None))
    ovout = np.zeros_like(vin)
    orc.oracle_xsph(pbfx.ptr(ovout), pbfx.ptr(vin), pbfx.ptr(pred), pbfx.ptr(a["is"]), pbfx.ptr(a["ks"]), C.byref(t),
                    C.byref(dp), n)
    sync(torch)
    np.testing.assert_array_equal(H(dvout), ovout)
    # aliasing is refused by the pbf_ entry point ...
    assert xs_fn(P(dvin), P(dvin), P(dpred), P(dg["is"]), P(dg["ks"]), *tab, C.byref(dp), n, None) == pbfx.PBF_ERR_INVALID
    # ... and made Jacobi by the reference-name one
    ref_fn = lib.LaunchXSPHCompact if hashed else lib.LaunchXSPH
    ref_fn.restype = None
    dvin2 = D(torch, vin)
    ref_fn(P(dvin2), P(dvin2), P(dpred), P(dg["is"]), P(dg["ks"]), *tab, dp, C.c_uint32(n), None)
    sync(torch)
    assert torch.equal(dvin2, dvout)


def test_integrate_boundary_velocity(gpu, lib, orc, scenes):
    torch = gpu
    p, pos, vel = scenes["compressed"]
    n = pos.shape[0]
    dpos, dvel = D(torch, pos), D(torch, vel)
    dpred = torch.empty_like(dpos)
    pbfx.check(lib.pbf_launch_integrate_pred(P(dpos), P(dvel), P(dpred), p.gravity, p.dt, n, None))
    opred = np.zeros_like(pos)
    orc.oracle_integrate_pred(pbfx.ptr(pos), pbfx.ptr(vel), pbfx.ptr(opred), p.gravity, p.dt, n)
    sync(torch)
    np.testing.assert_array_equal(H(dpred), opred)  # explicit FMA both sides: bit-exact
    pbfx.check(lib.pbf_launch_boundary(P(dpred), P(dvel), C.byref(p.grid), 0.3, n, None))
    ov = vel.copy()
    orc.oracle_boundary(pbfx.ptr(opred), pbfx.ptr(ov), C.byref(p.grid), 0.3, n)
    sync(torch)
    np.testing.assert_array_equal(H(dpred), opred)
    np.testing.assert_array_equal(H(dvel), ov)
    dv2 = torch.empty_like(dvel)
    pbfx.check(lib.pbf_launch_velocity(P(dv2), P(dpos), P(dpred), np.float32(1.0) / p.dt, n, None))
    ov2 = np.zeros_like(vel)
    orc.oracle_velocity(pbfx.ptr(ov2), pbfx.ptr(pos), pbfx.ptr(opred), np.float32(1.0) / p.dt, n)
    sync(torch)
    np.testing.assert_array_equal(H(dv2), ov2)


def test_bounded_wait_gives_up_and_context_survives(gpu, lib):
    torch = gpu
    scratch = torch.zeros(4, dtype=torch.int32, device="cuda")
    assert lib.pbf_selftest_bounded_wait(2000, P(scratch)) == pbfx.PBF_ERR_TIMEOUT
    # the context is still usable
    x = torch.arange(10, device="cuda").sum().item()
    assert x == 45


def test_stage_wait_gives_up_and_context_survives(gpu, lib):
    """The staging barrier's wait (TMA bulk copies into shared memory) is
    bounded: armed for bytes that never arrive, it records the timeout."""
    torch = gpu
    scratch = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.pbf_selftest_stage_wait(2000, P(scratch)) == pbfx.PBF_ERR_TIMEOUT
    x = torch.arange(10, device="cuda").sum().item()
    assert x == 45


def test_scorr_exponent_four_matches_runtime_powf_everywhere(gpu, lib):
    """The delta kernels' s_corr exponent n == 4 form equals powf(x, n) with n
    known only at run time, for every non-negative float (2.1e9 values)."""
    import ctypes as C

    mism, first = C.c_uint64(), C.c_uint32()
    pbfx.check(lib.pbf_selftest_powf4(C.byref(mism), C.byref(first)), "selftest_powf4")
    assert mism.value == 0, "first mismatch at bits 0x%08x" % first.value
