"""ctypes binding of libpbf_gb300 (include/pbf/pbf.h) and of the CPU oracle.

Host-side helper for tests, smoke() and bench.py: it only marshals arguments to
the C ABI.  The library is loaded from this package's lib/ directory; loading
fails loudly when it has not been built (there is no fallback path).
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG_DIR)
LIB_PATH = os.path.join(PKG_DIR, "lib", "libpbf_gb300.so")
ORACLE_PATH = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
REF_HARNESS_PATH = os.path.join(ROOT, "oracle", "_build", "libref_harness.so")
REF_IMAGES = os.path.join(ROOT, "oracle", "_ref")

PBF_OK = 0
PBF_ERR_INVALID = 1
PBF_ERR_CUDA = 2
PBF_ERR_OOM = 3
PBF_ERR_TIMEOUT = 4
PBF_ERR_NONFINITE = 5
PBF_ERR_UNSUPPORTED = 6
PBF_GRID_DENSE = 0
PBF_GRID_HASHED = 1
PBF_MATH_EXACT = 0
PBF_MATH_FAST = 1

DBG_KEYS_SORTED = 0
DBG_PERM = 1
DBG_CELL_START = 2
DBG_CELL_END = 3
DBG_UNIQUE_KEYS = 4
DBG_OFFSETS = 5
DBG_COMPACT_COUNT = 6
DBG_LAMBDA = 7
DBG_NUM_CELLS = 8


class Float3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Int3(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int)]


class KernelCoeffs(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("h", "inv_h", "h2", "poly6", "spiky", "visc")]


class GridBounds(C.Structure):
    _fields_ = [("mins", Float3), ("maxs", Float3), ("cellSize", C.c_float), ("dim", Int3)]


_TUNING = [
    ("scorr_enable", C.c_int), ("scorr_k", C.c_float), ("scorr_n", C.c_float), ("scorr_dq_h", C.c_float),
    ("wq_min", C.c_float), ("scorr_min", C.c_float), ("grad_r_eps", C.c_float), ("lambda_denom_eps", C.c_float),
    ("compliance", C.c_float), ("xpbd_enable", C.c_int), ("enable_lambda_clamp", C.c_int),
    ("lambda_max_abs", C.c_float), ("enable_disp_clamp", C.c_int), ("disp_clamp_max_h", C.c_float),
    ("enable_relax", C.c_int), ("relax_omega", C.c_float), ("xsph_gate_enable", C.c_int), ("xsph_n_min", C.c_int),
    ("xsph_n_max", C.c_int), ("lambda_warm_start_enable", C.c_int), ("lambda_warm_start_decay", C.c_float),
    ("semi_implicit_integration_enable", C.c_int),
]


class Tuning(C.Structure):
    _fields_ = _TUNING


class SimParams(C.Structure):
    _fields_ = [
        ("numParticles", C.c_uint32), ("maxParticles", C.c_uint32), ("gravity", Float3), ("dt", C.c_float),
        ("cfl", C.c_float), ("restDensity", C.c_float), ("solverIters", C.c_int), ("maxNeighbors", C.c_int),
        ("sortEveryN", C.c_int), ("boundaryRestitution", C.c_float), ("particleMass", C.c_float), ("pbf", Tuning),
        ("xsph_c", C.c_float), ("kernel", KernelCoeffs), ("grid", GridBounds), ("ghostParticleCount", C.c_uint32),
    ]


class DeviceParams(C.Structure):
    _fields_ = [
        ("kernel", KernelCoeffs), ("grid", GridBounds), ("gravity", Float3), ("restDensity", C.c_float),
        ("dt", C.c_float), ("inv_dt", C.c_float), ("boundaryRestitution", C.c_float), ("maxNeighbors", C.c_int),
        ("particleMass", C.c_float), ("pbf", Tuning), ("xsph_c", C.c_float),
    ]


class OracleTrace(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "keys", "keys_sorted", "perm", "cell_start", "cell_end", "unique_keys", "offsets", "compact_count",
        "lambda_", "pred_solved", "vel_pre_xsph")]


class OracleTable(C.Structure):
    _fields_ = [("start", C.c_void_p), ("end", C.c_void_p), ("unique_keys", C.c_void_p), ("offsets", C.c_void_p),
                ("count", C.c_uint32)]


def ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


_VP, _U32, _I, _F, _SZ = C.c_void_p, C.c_uint32, C.c_int, C.c_float, C.c_size_t

_SIGS = {
    "pbf_status_string": ([_I], C.c_char_p),
    "pbf_version": ([], _I),
    "pbf_abi_sizes": ([C.POINTER(C.c_uint32 * 5)], None),
    "pbf_default_tuning": ([C.POINTER(Tuning)], None),
    "pbf_make_kernel_coeffs": ([_F, C.POINTER(KernelCoeffs)], None),
    "pbf_make_device_params": ([C.POINTER(SimParams), C.POINTER(DeviceParams)], None),
    "pbf_compute_dims": ([C.POINTER(GridBounds), C.POINTER(C.c_int32 * 3)], None),
    "pbf_dam_break_params": ([_F, _F, _F, _I, _U32, C.POINTER(SimParams)], _I),
    "pbf_seed_lattice": ([_VP, _U32, _U32, _U32, _F, _F, _F, _F, _F, C.c_uint64, C.POINTER(GridBounds)], _I),
    "pbf_launch_integrate_pred": ([_VP, _VP, _VP, Float3, _F, _U32, _VP], _I),
    "pbf_launch_boundary": ([_VP, _VP, C.POINTER(GridBounds), _F, _U32, _VP], _I),
    "pbf_launch_velocity": ([_VP, _VP, _VP, _F, _U32, _VP], _I),
    "pbf_launch_hash_keys": ([_VP, _VP, _VP, C.POINTER(GridBounds), _U32, _VP], _I),
    "pbf_sort_pairs_query": ([C.POINTER(_SZ), _U32], _I),
    "pbf_launch_sort_pairs": ([_VP, _SZ, _VP, _VP, _VP, _VP, _U32, _VP], _I),
    "pbf_launch_sort_pairs_bits": ([_VP, _SZ, _VP, _VP, _VP, _VP, _U32, _I, _VP], _I),
    "pbf_launch_cell_ranges": ([_VP, _VP, _VP, _U32, _U32, _VP], _I),
    "pbf_cell_compact_scratch_query": ([C.POINTER(_SZ), _U32], _I),
    "pbf_launch_cell_ranges_compact": ([_VP, _SZ, _VP, _VP, _VP, _VP, _U32, _VP], _I),
    "pbf_launch_cell_ranges_compact_noalloc": ([_VP, _VP, _VP, _VP, _U32, _VP], _I),
    "pbf_launch_lambda": ([_VP, _VP, _VP, _VP, _VP, _VP, C.POINTER(DeviceParams), _U32, _VP], _I),
    "pbf_launch_lambda_compact": ([_VP, _VP, _VP, _VP, _VP, _VP, _VP, C.POINTER(DeviceParams), _U32, _VP], _I),
    "pbf_launch_delta_apply": ([_VP, _VP, _VP, _VP, _VP, _VP, _VP, C.POINTER(DeviceParams), _U32, _VP], _I),
    "pbf_launch_delta_apply_compact": ([_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, C.POINTER(DeviceParams), _U32, _VP],
                                       _I),
    "pbf_launch_xsph": ([_VP, _VP, _VP, _VP, _VP, _VP, _VP, C.POINTER(DeviceParams), _U32, _VP], _I),
    "pbf_launch_xsph_compact": ([_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, C.POINTER(DeviceParams), _U32, _VP], _I),
    "pbf_create": ([C.POINTER(SimParams), _I, C.POINTER(_VP)], _I),
    "pbf_destroy": ([_VP], _I),
    "pbf_stream": ([_VP], _VP),
    "pbf_set_stream": ([_VP, _VP], C.c_int),
    "pbf_device_state": ([_VP, C.POINTER(_VP), C.POINTER(_VP)], _I),
    "pbf_upload_state": ([_VP, _VP, _VP], _I),
    "pbf_download_state": ([_VP, _VP, _VP], _I),
    "pbf_step": ([_VP, C.POINTER(SimParams)], _I),
    "pbf_step_n": ([_VP, C.POINTER(SimParams), _I], _I),
    "pbf_step_host": ([_VP, C.POINTER(SimParams), _VP, _VP], _I),
    "pbf_synchronize": ([_VP], _I),
    "pbf_density_stats": ([_VP, C.POINTER(C.c_double * 4)], _I),
    "pbf_debug_fetch": ([_VP, _I, _VP, _SZ], _I),
    "pbf_selftest_bounded_wait": ([_U32, _VP], _I),
    "pbf_selftest_stage_wait": ([_U32, _VP], _I),
    "pbf_selftest_powf4": ([C.POINTER(C.c_uint64), C.POINTER(_U32)], _I),
    "pbf_debug_eval_math": ([_I, _VP, _VP, _VP, _U32], _I),
    "pbf_profile_step": ([_VP, C.POINTER(SimParams), C.POINTER(C.c_float), C.POINTER(C.c_char_p), _I,
                          C.POINTER(_I)], _I),
    "pbf_launches_per_step": ([_VP], _I),
    "pbf_set_neighbour_list_capacity": ([_VP, _U32], _I),
    "pbf_forward": ([_VP, _I, _I, C.POINTER(_VP)], _I),
    "pbf_backward": ([_VP, _VP, _VP, _VP, _VP, C.POINTER(_F)], _I),
    "pbf_tape_destroy": ([_VP], _I),
    "pbf_forward_batch": ([_VP, _I, _I, _I, _VP], _I),
    "pbf_backward_batch": ([_VP, _I, _VP, _VP, _VP, _VP, _VP], _I),
    "pbf_density_grid": ([_VP, _I, _VP], _I),
    "pbf_density_grid_loss": ([_VP, _I, _VP, C.POINTER(C.c_double), _VP], _I),
    "pbf_ensemble_create": ([C.POINTER(SimParams), _U32, C.POINTER(_VP)], _I),
    "pbf_ensemble_destroy": ([_VP], _I),
    "pbf_ensemble_stream": ([_VP], _VP),
    "pbf_ensemble_set_stream": ([_VP, _VP], C.c_int),
    "pbf_ensemble_num_particles": ([_VP], _U32),
    "pbf_ensemble_scene_offsets": ([_VP, _VP], _I),
    "pbf_ensemble_upload_state": ([_VP, _VP, _VP], _I),
    "pbf_ensemble_download_state": ([_VP, _VP, _VP], _I),
    "pbf_ensemble_step": ([_VP, _I], _I),
    "pbf_ensemble_step_host": ([_VP, _VP, _VP], _I),
    "pbf_ensemble_synchronize": ([_VP], _I),
    "pbf_ensemble_launches_per_step": ([_VP], _I),
    "pbf_neighbour_list_stats": ([_VP, C.POINTER(_U32), C.POINTER(_U32), C.POINTER(_U32), _I], _I),
    "pbf_console_create": ([C.POINTER(_VP)], _I),
    "pbf_console_destroy": ([_VP], _I),
    "pbf_console_set": ([_VP, C.c_char_p, C.c_double], _I),
    "pbf_console_get": ([_VP, C.c_char_p, C.POINTER(C.c_double)], _I),
    "pbf_console_prepare_cube_mix": ([_VP], _I),
    "pbf_console_merge_json": ([_VP, C.c_char_p, C.c_char_p, _U32], _I),
    "pbf_console_profile": ([_VP, C.c_char_p, _U32], _I),
    "pbf_console_build_sim_params": ([_VP, _I, C.POINTER(SimParams)], _I),
    "pbf_console_cube_mix_centers": ([_VP, C.POINTER(_F), _U32, C.POINTER(_U32)], _I),
    "pbf_seed_cube_mix": ([_VP, _VP], _I),
    "pbf_tile_shape_count": ([], _I),
    "pbf_tile_shape_info": ([_I, C.POINTER(_I), C.POINTER(_I)], _I),
    "pbf_set_tile_shape": ([_VP, _I], _I),
    "pbf_get_tile_shape": ([_VP, C.POINTER(_I)], _I),
    "pbf_autotune_tile_shape": ([_VP, C.POINTER(SimParams), _I, C.POINTER(_F), C.POINTER(_I)], _I),
    "pbf_ensemble_set_tile_shape": ([_VP, _I], _I),
    "pbf_ensemble_get_tile_shape": ([_VP, C.POINTER(_I)], _I),
    "pbf_ensemble_autotune": ([_VP, _I, C.POINTER(_F), C.POINTER(_I)], _I),
    "pbf_set_math_mode": ([_VP, _I], _I),
    "pbf_get_math_mode": ([_VP, C.POINTER(_I)], _I),
    "pbf_ensemble_set_math_mode": ([_VP, _I], _I),
    "pbf_ensemble_get_math_mode": ([_VP, C.POINTER(_I)], _I),
}

_ORACLE_SIGS = {
    "oracle_num_threads": ([], _I),
    "oracle_set_num_threads": ([_I], None),
    "oracle_integrate_pred": ([_VP, _VP, _VP, Float3, _F, _U32], None),
    "oracle_boundary": ([_VP, _VP, C.POINTER(GridBounds), _F, _U32], None),
    "oracle_velocity": ([_VP, _VP, _VP, _F, _U32], None),
    "oracle_hash_keys": ([_VP, _VP, _VP, C.POINTER(GridBounds), _U32], None),
    "oracle_sort_pairs": ([_VP, _VP, _VP, _VP, _U32], None),
    "oracle_cell_ranges": ([_VP, _VP, _VP, _U32, _U32], None),
    "oracle_cell_ranges_compact": ([_VP, _VP, _VP, _VP, _U32], None),
    "oracle_lambda": ([_VP, _VP, _VP, _VP, C.POINTER(OracleTable), C.POINTER(DeviceParams), _U32], None),
    "oracle_delta_apply": ([_VP, _VP, _VP, _VP, _VP, C.POINTER(OracleTable), C.POINTER(DeviceParams), _U32], None),
    "oracle_xsph": ([_VP, _VP, _VP, _VP, _VP, C.POINTER(OracleTable), C.POINTER(DeviceParams), _U32], None),
    "oracle_step_f32": ([C.POINTER(SimParams), _I, _VP, _VP, _U32, C.POINTER(OracleTrace)], _I),
    "oracle_step_f64": ([C.POINTER(SimParams), _I, _VP, _VP, _U32], _I),
    "oracle_density_stats_f32pos": ([C.POINTER(SimParams), _VP, _U32, C.POINTER(C.c_double * 4)], None),
    "oracle_density_stats_f64pos": ([C.POINTER(SimParams), _VP, _U32, C.POINTER(C.c_double * 4)], None),
    "oracle_step_jvp": ([C.POINTER(SimParams), _I, _I, _VP, _VP, _VP, _VP, C.c_double, _U32, _I], _I),
    "oracle_dam_break_params": ([_F, _F, _F, _I, _U32, C.POINTER(SimParams)], _I),
    "oracle_seed_lattice": ([_VP, _U32, _U32, _U32, _F, _F, _F, _F, _F, C.c_uint64, C.POINTER(GridBounds)], None),
}


def _bind(lib, sigs):
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


_REF_SIGS = {
    "ref_init": ([C.c_char_p], _I),
    "ref_error": ([], C.c_char_p),
    "ref_step": ([C.POINTER(SimParams), _I, _VP, _VP, _U32, C.POINTER(OracleTrace)], _I),
    "ref_time_steps": ([C.POINTER(SimParams), _I, _VP, _VP, _U32, _I, _I, C.POINTER(C.c_double)], _I),
    "ref_phase_lambda": ([_VP, _VP, _VP, _VP, C.POINTER(OracleTable), C.POINTER(DeviceParams), _U32, _U32], _I),
    "ref_phase_delta_apply": ([_VP, _VP, _VP, _VP, _VP, C.POINTER(OracleTable), C.POINTER(DeviceParams), _U32, _U32],
                              _I),
    "ref_phase_xsph": ([_VP, _VP, _VP, _VP, _VP, C.POINTER(OracleTable), C.POINTER(DeviceParams), _U32, _U32], _I),
    "ref_phase_integrate_boundary": ([_VP, _VP, _VP, C.POINTER(SimParams), _U32], _I),
}

_lib = None
_oracle = None
_ref = None


def load(path: str = LIB_PATH):
    """The CUDA library.  Raises if it is missing (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError("libpbf_gb300.so not built: run __graft_entry__.build()")
        _lib = _bind(C.CDLL(path), _SIGS)
    return _lib


def load_oracle(path: str = ORACLE_PATH):
    """The CPU oracle (test infrastructure only)."""
    global _oracle
    if _oracle is None:
        if not os.path.exists(path):
            raise RuntimeError("oracle not built: run __graft_entry__.build()")
        _oracle = _bind(C.CDLL(path), _ORACLE_SIGS)
    return _oracle


def load_ref():
    """The reference's own kernels driven by oracle/ref/ref_harness.cu (test
    infrastructure only), or None when its device images are not present."""
    global _ref
    if _ref is None:
        imgs = os.path.join(REF_IMAGES, "pbf_lambda.cubin")
        if not (os.path.exists(REF_HARNESS_PATH) and os.path.exists(imgs)):
            return None
        lib = _bind(C.CDLL(REF_HARNESS_PATH), _REF_SIGS)
        if lib.ref_init(REF_IMAGES.encode()) != 0:
            raise RuntimeError("reference harness: %s" % lib.ref_error().decode())
        _ref = lib
    return _ref


def check(status: int, what: str = "call"):
    if status != PBF_OK:
        msg = load().pbf_status_string(status).decode()
        raise RuntimeError("%s failed: %d (%s)" % (what, status, msg))


def dam_break_params(box, iters: int = 2, num_particles: int = 0) -> SimParams:
    p = SimParams()
    check(load().pbf_dam_break_params(box[0], box[1], box[2], iters, num_particles, C.byref(p)), "dam_break_params")
    return p


def oracle_dam_break_params(orc, box, iters: int = 2, num_particles: int = 0) -> SimParams:
    """dam_break_params from the oracle's restatement (no product library)."""
    p = SimParams()
    if orc.oracle_dam_break_params(box[0], box[1], box[2], iters, num_particles, C.byref(p)) != 0:
        raise ValueError("invalid dam-break box or iteration count")
    return p


def oracle_seed_lattice(orc, nx, ny, nz, origin, spacing, jitter, seed, params: SimParams) -> np.ndarray:
    """seed_lattice from the oracle's restatement (no product library)."""
    out = np.zeros((nx * ny * nz, 4), dtype=np.float32)
    orc.oracle_seed_lattice(ptr(out), nx, ny, nz, origin[0], origin[1], origin[2], spacing, jitter, seed,
                            C.byref(params.grid))
    return out


def device_params(p: SimParams) -> DeviceParams:
    d = DeviceParams()
    load().pbf_make_device_params(C.byref(p), C.byref(d))
    return d


def num_cells(p: SimParams) -> int:
    return int(p.grid.dim.x) * int(p.grid.dim.y) * int(p.grid.dim.z)


def seed_lattice(lib, nx, ny, nz, origin, spacing, jitter, seed, params: SimParams) -> np.ndarray:
    out = np.zeros((nx * ny * nz, 4), dtype=np.float32)
    check(lib.pbf_seed_lattice(ptr(out), nx, ny, nz, origin[0], origin[1], origin[2], spacing, jitter, seed,
                               C.byref(params.grid)), "seed_lattice")
    return out


def rel_err(a, b, floor_frac: float = 1e-2) -> float:
    """max_i |a_i - b_i| / max(|b_i|, floor_frac * max_j |b_j|)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if b.size == 0:
        return 0.0
    scale = np.max(np.abs(b))
    floor = floor_frac * scale if scale > 0 else 1e-30
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def assert_close(a, b, tol: float, what: str, floor_frac: float = 1e-2):
    e = rel_err(a, b, floor_frac)
    if not e <= tol:
        raise AssertionError("%s: relative error %.3e > %.1e" % (what, e, tol))


class Sim:
    """Owning wrapper of a pbf_sim handle."""

    def __init__(self, lib, params: SimParams, hashed: bool = True):
        self.lib = lib
        self.params = params
        self.h = C.c_void_p()
        check(lib.pbf_create(C.byref(params), PBF_GRID_HASHED if hashed else PBF_GRID_DENSE, C.byref(self.h)),
              "pbf_create")
        self.n = int(params.numParticles)

    def close(self):
        if self.h:
            self.lib.pbf_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, pos: np.ndarray, vel: np.ndarray):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        vel = np.ascontiguousarray(vel, dtype=np.float32)
        assert pos.shape == (self.n, 4) and vel.shape == (self.n, 4)
        check(self.lib.pbf_upload_state(self.h, ptr(pos), ptr(vel)), "upload")

    def download(self):
        pos = np.zeros((self.n, 4), np.float32)
        vel = np.zeros((self.n, 4), np.float32)
        check(self.lib.pbf_download_state(self.h, ptr(pos), ptr(vel)), "download")
        return pos, vel

    def step(self, n: int = 1, params: SimParams | None = None):
        check(self.lib.pbf_step_n(self.h, C.byref(params) if params is not None else None, n), "step")
        check(self.lib.pbf_synchronize(self.h), "synchronize")

    def fetch(self, item: int):
        if item in (DBG_CELL_START, DBG_CELL_END):
            cnt = num_cells(self.params)
        elif item == DBG_OFFSETS:
            cnt = self.n + 1
        elif item in (DBG_COMPACT_COUNT, DBG_NUM_CELLS):
            cnt = 1
        else:
            cnt = self.n
        dt = np.float32 if item == DBG_LAMBDA else np.uint32
        out = np.zeros(cnt, dtype=dt)
        check(self.lib.pbf_debug_fetch(self.h, item, ptr(out), out.nbytes), "debug_fetch")
        return out

    def profile_step(self, params: SimParams | None = None):
        ms = (C.c_float * 32)()
        names = (C.c_char_p * 32)()
        cnt = C.c_int()
        check(self.lib.pbf_profile_step(self.h, C.byref(params) if params is not None else None, ms, names, 32,
                                        C.byref(cnt)), "profile_step")
        return [(names[k].decode(), float(ms[k])) for k in range(cnt.value)]

    def launches_per_step(self) -> int:
        return int(self.lib.pbf_launches_per_step(self.h))

    def set_list_capacity(self, entries: int):
        check(self.lib.pbf_set_neighbour_list_capacity(self.h, entries), "set_neighbour_list_capacity")

    def set_tile_shape(self, shape: int):
        check(self.lib.pbf_set_tile_shape(self.h, shape), "set_tile_shape")

    def set_math_mode(self, mode: int):
        check(self.lib.pbf_set_math_mode(self.h, mode), "set_math_mode")

    def math_mode(self) -> int:
        v = _I()
        check(self.lib.pbf_get_math_mode(self.h, C.byref(v)), "get_math_mode")
        return int(v.value)

    def tile_shape(self) -> int:
        v = _I()
        check(self.lib.pbf_get_tile_shape(self.h, C.byref(v)), "get_tile_shape")
        return int(v.value)

    def autotune(self, steps: int = 3, params: SimParams | None = None):
        """Runs the tile-shape autotuner; returns (chosen shape, ms per step of each shape)."""
        n = int(self.lib.pbf_tile_shape_count())
        ms = (_F * n)()
        chosen = _I()
        check(self.lib.pbf_autotune_tile_shape(self.h, C.byref(params) if params is not None else None, steps, ms,
                                               C.byref(chosen)), "autotune_tile_shape")
        return int(chosen.value), [float(x) for x in ms]

    def list_stats(self, reset: bool = False):
        """(capacity, longest list, overflowed lists) since the last reset."""
        c, l, o = _U32(), _U32(), _U32()
        check(self.lib.pbf_neighbour_list_stats(self.h, C.byref(c), C.byref(l), C.byref(o), int(reset)),
              "neighbour_list_stats")
        return int(c.value), int(l.value), int(o.value)

    def stream_ptr(self) -> int:
        return int(self.lib.pbf_stream(self.h) or 0)

    def set_stream(self, stream: int | None):
        """Enqueue on a caller's cudaStream_t (an int); None: the handle's own stream."""
        check(self.lib.pbf_set_stream(self.h, C.c_void_p(stream or None)), "set_stream")

    def density_stats(self):
        out = (C.c_double * 4)()
        check(self.lib.pbf_density_stats(self.h, C.byref(out)), "density_stats")
        return list(out)


def forward_batch(lib, sims, steps: int, every: int):
    """pbf_forward_batch over Sim objects; returns their tapes (c_void_p)."""
    k = len(sims)
    tapes = (_VP * k)()
    check(lib.pbf_forward_batch((_VP * k)(*[s.h.value for s in sims]), k, steps, every, tapes), "forward_batch")
    return [C.c_void_p(t) for t in tapes]


def backward_batch(lib, tapes, pos_bar, vel_bar, pos0_bar=None, vel0_bar=None):
    """pbf_backward_batch; the *_bar arguments are lists of device pointers
    (ints), one per scene; returns dL/d(xsph_c) of each scene."""
    k = len(tapes)

    def arr(v):
        return None if v is None else (_VP * k)(*v)

    cb = (_F * k)()
    check(lib.pbf_backward_batch((_VP * k)(*[t.value for t in tapes]), k, arr(pos_bar), arr(vel_bar), arr(pos0_bar),
                                 arr(vel0_bar), cb), "backward_batch")
    return [float(x) for x in cb]


class Ensemble:
    """Owning wrapper of a pbf_ensemble handle (scenes: a list of SimParams)."""

    def __init__(self, lib, scenes):
        self.lib = lib
        arr = (SimParams * len(scenes))(*scenes)
        self.h = C.c_void_p()
        check(lib.pbf_ensemble_create(arr, len(scenes), C.byref(self.h)), "pbf_ensemble_create")
        self.n = int(lib.pbf_ensemble_num_particles(self.h))
        self.offsets = np.zeros(len(scenes) + 1, np.uint32)
        check(lib.pbf_ensemble_scene_offsets(self.h, ptr(self.offsets)), "scene_offsets")

    def close(self):
        if self.h:
            self.lib.pbf_ensemble_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, pos: np.ndarray, vel: np.ndarray):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        vel = np.ascontiguousarray(vel, dtype=np.float32)
        assert pos.shape == (self.n, 4) and vel.shape == (self.n, 4)
        check(self.lib.pbf_ensemble_upload_state(self.h, ptr(pos), ptr(vel)), "ensemble upload")

    def download(self):
        pos = np.zeros((self.n, 4), np.float32)
        vel = np.zeros((self.n, 4), np.float32)
        check(self.lib.pbf_ensemble_download_state(self.h, ptr(pos), ptr(vel)), "ensemble download")
        return pos, vel

    def step(self, n: int = 1):
        check(self.lib.pbf_ensemble_step(self.h, n), "ensemble step")
        check(self.lib.pbf_ensemble_synchronize(self.h), "ensemble synchronize")

    def stream_ptr(self) -> int:
        return int(self.lib.pbf_ensemble_stream(self.h) or 0)

    def set_stream(self, stream: int | None):
        """Enqueue on a caller's cudaStream_t (an int); None: the ensemble's own stream."""
        check(self.lib.pbf_ensemble_set_stream(self.h, C.c_void_p(stream or None)), "ensemble set_stream")

    def launches_per_step(self) -> int:
        return int(self.lib.pbf_ensemble_launches_per_step(self.h))

    def set_tile_shape(self, shape: int):
        check(self.lib.pbf_ensemble_set_tile_shape(self.h, shape), "ensemble set_tile_shape")

    def set_math_mode(self, mode: int):
        check(self.lib.pbf_ensemble_set_math_mode(self.h, mode), "ensemble set_math_mode")

    def tile_shape(self) -> int:
        v = _I()
        check(self.lib.pbf_ensemble_get_tile_shape(self.h, C.byref(v)), "ensemble get_tile_shape")
        return int(v.value)

    def autotune(self, steps: int = 3):
        """Runs the tile-shape autotuner; returns (chosen shape, ms per step of each shape)."""
        n = int(self.lib.pbf_tile_shape_count())
        ms = (_F * n)()
        chosen = _I()
        check(self.lib.pbf_ensemble_autotune(self.h, steps, ms, C.byref(chosen)), "ensemble autotune")
        return int(chosen.value), [float(x) for x in ms]


class Console:
    """Owning wrapper of a pbf_console: the reference application's runtime
    configuration (RuntimeConsole) and its mapping to SimParams.  Fields are
    read and written by name, e.g. con["sim.particleRadiusWorld"] = 0.005."""

    def __init__(self, lib):
        self.lib = lib
        self.h = _VP()
        check(lib.pbf_console_create(C.byref(self.h)), "console_create")

    def close(self):
        if self.h:
            self.lib.pbf_console_destroy(self.h)
            self.h = _VP()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __getitem__(self, field: str) -> float:
        v = C.c_double()
        check(self.lib.pbf_console_get(self.h, field.encode(), C.byref(v)), "console_get " + field)
        return float(v.value)

    def __setitem__(self, field: str, value: float):
        check(self.lib.pbf_console_set(self.h, field.encode(), float(value)), "console_set " + field)

    def prepare_cube_mix(self):
        check(self.lib.pbf_console_prepare_cube_mix(self.h), "console_prepare_cube_mix")

    def merge_json(self, text: str):
        """Merges a config.json text; raises ValueError (console unchanged) if it is rejected."""
        err = C.create_string_buffer(512)
        if self.lib.pbf_console_merge_json(self.h, text.encode(), err, len(err)) != PBF_OK:
            raise ValueError(err.value.decode())

    def profile(self) -> str:
        buf = C.create_string_buffer(256)
        check(self.lib.pbf_console_profile(self.h, buf, len(buf)), "console_profile")
        return buf.value.decode()

    def sim_params(self, sanitize: bool = True) -> SimParams:
        p = SimParams()
        check(self.lib.pbf_console_build_sim_params(self.h, int(sanitize), C.byref(p)), "console_build_sim_params")
        return p

    def cube_mix_centers(self) -> np.ndarray:
        n = _U32()
        check(self.lib.pbf_console_cube_mix_centers(self.h, None, 0, C.byref(n)), "console_cube_mix_centers")
        out = np.zeros((n.value, 3), np.float32)
        if n.value:
            check(self.lib.pbf_console_cube_mix_centers(self.h, out.ctypes.data_as(C.POINTER(_F)), n.value,
                                                        C.byref(n)), "console_cube_mix_centers")
        return out


def tile_shapes(lib):
    """[(particles per CTA, staged slots)] of the neighbour passes' tile shapes."""
    out = []
    for i in range(int(lib.pbf_tile_shape_count())):
        t, st = _I(), _I()
        check(lib.pbf_tile_shape_info(i, C.byref(t), C.byref(st)), "tile_shape_info")
        out.append((int(t.value), int(st.value)))
    return out


def lattice_dims(total: int, box_extent, spacing: float):
    """Lattice (nx, ny, nz) holding `total` particles packed from the min
    corner of a box, as Simulator::seedBoxLatticeAuto chooses it
    (sim/simulator.cpp:880-934)."""
    cap = [max(1, int(math.floor(e / spacing))) for e in box_extent]
    t = max(1, total)
    nx = min(cap[0], int(math.ceil(t ** (1.0 / 3.0))))
    rem = (t + nx - 1) // nx
    ny = min(cap[1], int(math.ceil(math.sqrt(rem))))
    nz = min(cap[2], int(math.ceil(rem / max(1, ny))))
    while nx * ny * nz < t:
        if nx < cap[0]:
            nx += 1
        elif ny < cap[1]:
            ny += 1
        elif nz < cap[2]:
            nz += 1
        else:
            break
    return nx, ny, nz


def ensemble_scenes(lib, num_scenes: int, seed: int = 0xE45E, n_min: int = 2048, n_max: int = 65536,
                    iters_choices=(2, 3)):
    """Seeded batch of dam-break scenes: N_s = round(exp(U[ln n_min, ln n_max])),
    box extents U[0.3, 1.0]^3 m, gravity 9.8 m/s^2 tilted from -y by up to 15
    degrees in a uniform direction, solver iterations drawn from iters_choices,
    a block of N_s lattice particles at spacing 0.01 (jitter +-0.0005) packed
    from the box's min corner (a box that cannot hold N_s particles at that
    spacing is filled: fewer particles).  Returns (list of SimParams,
    concatenated pos)."""
    rng = np.random.default_rng(seed)
    scenes, blocks = [], []
    for s in range(num_scenes):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        ext = rng.uniform(0.3, 1.0, 3)
        iters = int(rng.choice(iters_choices))
        p = dam_break_params(tuple(float(e) for e in ext), iters, n)
        theta = math.radians(rng.uniform(0.0, 15.0))
        phi = rng.uniform(0.0, 2.0 * math.pi)
        g = 9.8
        p.gravity = Float3(g * math.sin(theta) * math.cos(phi), -g * math.cos(theta), g * math.sin(theta) * math.sin(phi))
        nx, ny, nz = lattice_dims(n, ext, 0.01)
        # a box too small for N_s particles at this spacing is filled instead
        n = min(n, nx * ny * nz)
        pos = seed_lattice(lib, nx, ny, nz, (0.005, 0.005, 0.005), 0.01, 0.0005, seed * 1000003 + s, p)[:n]
        p.numParticles = p.maxParticles = n
        scenes.append(p)
        blocks.append(pos)
    return scenes, np.ascontiguousarray(np.concatenate(blocks))


def oracle_step(orc, params: SimParams, hashed: bool, pos: np.ndarray, vel: np.ndarray, trace: bool = True):
    """One FP32 oracle step in place; returns the trace arrays."""
    return _traced_step(orc.oracle_step_f32, params, hashed, pos, vel, trace)


def ref_step(ref, params: SimParams, hashed: bool, pos: np.ndarray, vel: np.ndarray, trace: bool = True):
    """One step of the reference's own kernels in place; returns the trace
    (keys, sorted keys, permutation, cell tables, lambda)."""
    return _traced_step(ref.ref_step, params, hashed, pos, vel, trace, gpu_ref=True)


def _traced_step(fn, params, hashed, pos, vel, trace, gpu_ref=False):
    n = int(pos.shape[0])
    nc = num_cells(params)
    tr = {}
    t = OracleTrace()
    if trace:
        tr = {
            "keys": np.zeros(n, np.uint32), "keys_sorted": np.zeros(n, np.uint32), "perm": np.zeros(n, np.uint32),
            "lambda": np.zeros(n, np.float32), "pred_solved": np.zeros((n, 4), np.float32),
            "vel_pre_xsph": np.zeros((n, 4), np.float32),
        }
        if hashed:
            tr["unique_keys"] = np.zeros(max(n, 1), np.uint32)
            tr["offsets"] = np.zeros(n + 1, np.uint32)
            tr["compact_count"] = np.zeros(1, np.uint32)
        else:
            tr["cell_start"] = np.zeros(nc, np.uint32)
            tr["cell_end"] = np.zeros(nc, np.uint32)
        for k, v in tr.items():
            setattr(t, "lambda_" if k == "lambda" else k, v.ctypes.data)
    if gpu_ref:
        t.pred_solved = None
        t.vel_pre_xsph = None
        tr.pop("pred_solved", None)
        tr.pop("vel_pre_xsph", None)
    rc = fn(C.byref(params), 1 if hashed else 0, ptr(pos), ptr(vel), n, C.byref(t) if trace else None)
    if rc != 0:
        raise RuntimeError("step failed (%d)" % rc)
    if trace and hashed:
        m = int(tr["compact_count"][0])
        tr["unique_keys"] = tr["unique_keys"][:m]
        tr["offsets"] = tr["offsets"][: m + 1]
    return tr
