"""ctypes binding of librebound_gb300.so (the C ABI in include/rebound_gb300.h).

The shared library is built in-tree by rebound_gb300.build.  Importing this
module loads it and fails loudly if it cannot: there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librebound_gb300.so")

# struct reb_particle (src/rebound.h:86-104), 112 bytes.
PARTICLE_DTYPE = np.dtype([
    ("x", "f8"), ("y", "f8"), ("z", "f8"), ("vx", "f8"), ("vy", "f8"), ("vz", "f8"),
    ("ax", "f8"), ("ay", "f8"), ("az", "f8"), ("m", "f8"), ("r", "f8"),
    ("name", "u8"), ("ap", "u8"), ("sim", "u8")])
# struct reb_collision (src/rebound.h:144-149), 72 bytes.
COLLISION_DTYPE = np.dtype([("p1", "u8"), ("p2", "u8"), ("gb", "f8", 6), ("ri", "u8")])
# Tree cell export record (rgpu_tree_export), 88 bytes.
CELL_DTYPE = np.dtype([("root", "i4"), ("depth", "i4"), ("path", "u8"), ("x", "f8"), ("y", "f8"), ("z", "f8"),
                       ("w", "f8"), ("m", "f8"), ("mx", "f8"), ("my", "f8"), ("mz", "f8"), ("pt", "i8")])

RGPU_OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "unsupported",
          5: "non-finite particle", 6: "particle outside box", 7: "duplicate positions in tree",
          8: "tree too deep", 9: "output overflow", 10: "capacity exceeded", 11: "timeout"}

GRAVITY = {"none": 0, "basic": 1, "compensated": 2, "tree": 3, "mixed": 64, "mixed_split": 65, "tree_split": 66}
COLLISION = {"none": 0, "direct": 1, "tree": 2, "line": 4, "linetree": 5}
BOUNDARY = {"none": 0, "open": 1, "periodic": 2, "shear": 3}
INTEGRATOR = {"leapfrog": 0, "sei": 1, "whfast": 2}
RESOLVE = {"halt": 0, "hardsphere": 1, "none": 2}


class Config(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in (
        "G", "softening", "dt", "t", "OMEGA", "OMEGAZ", "root_size", "opening_angle2",
        "coefficient_of_restitution", "minimum_collision_velocity")] + [
        ("N_active", ctypes.c_int64), ("testparticle_type", ctypes.c_int32),
        ("gravity_ignore_terms", ctypes.c_int32),
        ("N_root_x", ctypes.c_int32), ("N_root_y", ctypes.c_int32), ("N_root_z", ctypes.c_int32),
        ("N_ghost_x", ctypes.c_int32), ("N_ghost_y", ctypes.c_int32), ("N_ghost_z", ctypes.c_int32),
        ("gravity", ctypes.c_int32), ("collision", ctypes.c_int32), ("collision_resolve", ctypes.c_int32),
        ("boundary", ctypes.c_int32), ("integrator", ctypes.c_int32), ("whfast_safe_mode", ctypes.c_int32),
        ("rand_seed", ctypes.c_uint32), ("status", ctypes.c_int32), ("collisions_log_n", ctypes.c_int64),
        ("leapfrog_order", ctypes.c_int32), ("whfast_coordinates", ctypes.c_int32),
        ("whfast_corrector", ctypes.c_int32), ("whfast_corrector2", ctypes.c_int32),
        ("whfast_kernel", ctypes.c_int32), ("whfast_keep_unsynchronized", ctypes.c_int32),
        ("exact_finish_time", ctypes.c_int32), ("tree_quadrupole", ctypes.c_int32),
        ("collisions_plog", ctypes.c_double)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("steps_per_launch", ctypes.c_int64),
                ("slots_per_bucket", ctypes.c_int32), ("pool_particles", ctypes.c_int32),
                ("cluster_steps_per_tick", ctypes.c_int32), ("thread_per_system", ctypes.c_int32),
                ("tick_ns", ctypes.c_int64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_int64), ("waiting", ctypes.c_int64), ("resident", ctypes.c_int64),
                ("ticks", ctypes.c_int64), ("system_steps", ctypes.c_double),
                ("pair_interactions", ctypes.c_double), ("bytes_in_use", ctypes.c_size_t)]


class RGPUError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"rebound_gb300 error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


_lib = None

# Every exported entry point with (restype, argtypes).
_P = ctypes.c_void_p
SIGNATURES = {
    "rgpu_config_default": (None, [ctypes.POINTER(Config)]),
    "rgpu_sim_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p)]),
    "rgpu_sim_free": (None, [_P]),
    "rgpu_sim_last_error": (ctypes.c_char_p, [_P]),
    "rgpu_sim_configure": (ctypes.c_int, [_P, ctypes.POINTER(Config)]),
    "rgpu_sim_get_config": (ctypes.c_int, [_P, ctypes.POINTER(Config)]),
    "rgpu_sim_set_restitution_fn": (ctypes.c_int, [_P, _P, _P]),
    "rgpu_sim_resolve_time": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]),
    "rgpu_sim_set_particles": (ctypes.c_int, [_P, _P, ctypes.c_size_t, ctypes.c_size_t]),
    "rgpu_sim_get_particles": (ctypes.c_int, [_P, _P, ctypes.c_size_t, ctypes.c_size_t]),
    "rgpu_sim_N": (ctypes.c_size_t, [_P]),
    "rgpu_update_acceleration": (ctypes.c_int, [_P]),
    "rgpu_collision_search": (ctypes.c_int, [_P, _P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "rgpu_tree_export": (ctypes.c_int, [_P, _P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "rgpu_steps": (ctypes.c_int, [_P, ctypes.c_int64]),
    "rgpu_integrate": (ctypes.c_int, [_P, ctypes.c_double]),
    "rgpu_synchronize": (ctypes.c_int, [_P]),
    "rgpu_energy": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double)]),
    "rgpu_sim_sync": (ctypes.c_int, [_P]),
    "rgpu_sim_snapshot_size": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "rgpu_sim_snapshot_write": (ctypes.c_int, [_P, _P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "rgpu_sim_snapshot_read": (ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    "rgpu_sim_save_to_file": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_double, ctypes.c_int64, ctypes.c_int]),
    "rgpu_archive_scan": (ctypes.c_int, [ctypes.c_char_p, _P, _P, ctypes.c_size_t,
                                         ctypes.POINTER(ctypes.c_size_t)]),
    "rgpu_sim_load_from_file": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int64]),
    "rgpu_sim_last_kernel_ms": (ctypes.c_double, [_P]),
    "rgpu_launch_count": (ctypes.c_int64, []),
    "rgpu_sim_kernel_timer": (ctypes.c_int, [_P, ctypes.c_int]),
    "rgpu_sim_kernel_time": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]),
    "rgpu_sim_time_steps": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(ctypes.c_double)]),
    "rgpu_l2_flush": (ctypes.c_int, [_P, ctypes.c_size_t]),
    "rgpu_set_kernel_variant": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "rgpu_set_displacement_mode": (ctypes.c_int, [ctypes.c_int]),
    "rgpu_sim_guard_stats": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "rgpu_probe_rate": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "rgpu_selftest_exactfp": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_longlong)]),
    "rgpu_selftest_fastmath": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_double)]),
    "rgpu_direct_accel_noalloc": (ctypes.c_int, [_P] * 7 + [ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                                            ctypes.c_int, _P]),
    "rgpu_kepler_solve": (ctypes.c_int, [_P, ctypes.c_size_t, _P, _P, _P, ctypes.c_size_t]),
    "rgpu_ensemble_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), _P, ctypes.c_size_t, _P,
                                            ctypes.c_size_t, _P, ctypes.c_double, ctypes.c_int]),
    "rgpu_ensemble_free": (None, [_P]),
    "rgpu_ensemble_last_error": (ctypes.c_char_p, [_P]),
    "rgpu_ensemble_set_launch": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int64]),
    "rgpu_ensemble_set_mapping": (ctypes.c_int, [_P, ctypes.c_int]),
    "rgpu_ensemble_get_launch": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_int64)]),
    "rgpu_ensemble_steps": (ctypes.c_int, [_P, ctypes.c_int64]),
    "rgpu_ensemble_time_steps": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(ctypes.c_double)]),
    "rgpu_ensemble_autotune": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_double)]),
    "rgpu_ensemble_get_particles": (ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    "rgpu_ensemble_energy": (ctypes.c_int, [_P, _P]),
    "rgpu_ensemble_times": (ctypes.c_int, [_P, _P]),
    "rgpu_server_config_default": (None, [ctypes.POINTER(ServerConfig)]),
    "rgpu_server_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ServerConfig)]),
    "rgpu_server_free": (None, [_P]),
    "rgpu_server_submit": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_double,
                                          ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                          ctypes.POINTER(ctypes.c_int64)]),
    "rgpu_server_wait": (ctypes.c_int, [_P, ctypes.c_int64, _P, ctypes.c_size_t, ctypes.c_double,
                                        ctypes.POINTER(ctypes.c_double)]),
    "rgpu_server_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(ServerStats)]),
    "rgpu_ic_plummer": (ctypes.c_int, [ctypes.c_uint, ctypes.c_size_t, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, _P, ctypes.c_size_t]),
    "rgpu_ic_ring_patch": (ctypes.c_int, [ctypes.c_uint] + [ctypes.c_double] * 10 +
                           [_P, ctypes.c_size_t, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "rgpu_ic_planetary": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint), ctypes.c_int] + [ctypes.c_double] * 8 +
                          [_P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_double)]),
}
# Optional entry points bound when the library exports them.
OPTIONAL = {}


def load(build_if_missing=True):
    """Load the CUDA library (building it with nvcc if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _b
    if not _b.elf_matches_host(LIB_PATH):
        if not build_if_missing:
            raise ImportError(f"{LIB_PATH} is missing; run rebound_gb300.build.build()")
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    for name, (res, args) in OPTIONAL.items():
        if hasattr(L, name):
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
    _lib = L
    return L


def check(rc, handle=None):
    if rc != RGPU_OK:
        msg = ""
        if handle:
            raw = load().rgpu_sim_last_error(handle)
            msg = raw.decode() if raw else ""
        raise RGPUError(rc, msg)
