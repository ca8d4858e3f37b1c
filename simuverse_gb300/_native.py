"""ctypes binding of liblbm.so (include/lbm.h).

The library must have been built (``simuverse_gb300.build.build()`` or
``__graft_entry__.build()``); there is no fallback implementation, and loading fails
loudly when the shared object is missing.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# SIMUVERSE_LBM_VARIANT=bounds loads the bounds-checked build (liblbm_bounds.so) instead
VARIANT = os.environ.get("SIMUVERSE_LBM_VARIANT") or None
LIB_PATH = os.path.join(HERE, "_lib", "liblbm_bounds.so" if VARIANT == "bounds" else "liblbm.so")

# status codes (lbm.h)
LBM_OK = 0
LBM_IGNORED = 1
LBM_ERR_ARG = -1
LBM_ERR_CUDA = -2
LBM_ERR_TIMEOUT = -3
LBM_ERR_NAN = -4
LBM_ERR_IO = -5
LBM_ERR_STATE = -6
LBM_ERR_NOMEM = -7

MODES = {"reference": 0, "physics": 1}
DTYPES = {"f32": 0, "f64": 1, "f16": 2, "bf16": 3}
SCENES = {"poiseuille": 0, "cavity": 1, "custom": 2, "channel": 3, "periodic": 4}
KERNELS = {"auto": 0, "cell": 1, "vec4": 2, "bulk": 3, "vec2": 4, "tiled": 5, "ring": 6}
COLLISIONS = {"bgk": 0, "regularized": 1, "mrt": 2, "kbc": 3}
ROUNDINGS = {"nearest": 0, "stochastic": 1}
ARITHS = {"exact": 0, "fast": 1}
BULK, BOUNDARY, INLET, OBSTACLE, OUTLET, EXTERNAL_FORCE, GHOST = 1, 2, 3, 4, 5, 6, 7

# LatticeInfo (simuverse/src/fluid/lattice.rs:5-13)
INFO_DTYPE = np.dtype([("material", "<i4"), ("block_iter", "<i4"), ("vx", "<f4"), ("vy", "<f4")])


class LbmParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
        ("mode", ctypes.c_int32), ("dtype", ctypes.c_int32), ("scene", ctypes.c_int32),
        ("tau", ctypes.c_float), ("lid_speed", ctypes.c_float), ("inlet_speed", ctypes.c_float),
        ("solid_fraction", ctypes.c_float), ("disk_rmin", ctypes.c_float), ("disk_rmax", ctypes.c_float),
        ("seed", ctypes.c_uint64),
        ("pixel_size", ctypes.c_int32), ("macro_every_step", ctypes.c_int32),
        ("kernel", ctypes.c_int32), ("collision", ctypes.c_int32), ("rounding", ctypes.c_int32),
        ("arith", ctypes.c_int32), ("reserved", ctypes.c_int32 * 2),
    ]


class ParticleParams(ctypes.Structure):
    _fields_ = [("canvas_w", ctypes.c_int32), ("canvas_h", ctypes.c_int32), ("count", ctypes.c_int32),
                ("life_time", ctypes.c_float), ("point_size", ctypes.c_int32), ("speed_factor", ctypes.c_float),
                ("fade_out_factor", ctypes.c_float), ("color_ty", ctypes.c_int32), ("color", ctypes.c_float * 4),
                ("seed", ctypes.c_uint64), ("deterministic", ctypes.c_int32), ("reserved", ctypes.c_int32 * 3)]


COLOR_MODES = {"curl": 0, "angle": 1}


class Edit(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("a", ctypes.c_float), ("b", ctypes.c_float), ("c", ctypes.c_float),
                ("d", ctypes.c_float)]


EDITS = {"obstacle": 0, "click": 1, "force": 2, "touch_begin": 3, "touch_move": 4}


class DomainDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("scene", ctypes.c_int32),
                ("tau", ctypes.c_float), ("speed", ctypes.c_float), ("reserved", ctypes.c_int32 * 3)]


class BatchConfig(ctypes.Structure):
    _fields_ = [("tile_threads_x", ctypes.c_int32), ("tile_rows", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("method", ctypes.c_int32),
                ("ms_per_step", ctypes.c_float), ("cells_per_thread", ctypes.c_int32),
                ("linear", ctypes.c_int32), ("full_occupancy", ctypes.c_int32)]


BATCH_METHODS = {"persistent": 0, "tile_launches": 1, "domain_loop": 2}


class LbmError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__("lbm error %d: %s" % (code, message))
        self.code = code


_P = ctypes.c_void_p
_I = ctypes.c_int32
_F = ctypes.c_float
_D = ctypes.c_double

# name -> argtypes; every function returns int
_SIGNATURES = {
    "lbm_memory_set_retain": [ctypes.c_uint64],
    "lbm_memory_trim": [],
    "lbm_memory_stats": [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)],
    "lbm_create": [ctypes.POINTER(LbmParams), ctypes.POINTER(_P)],
    "lbm_destroy": [_P],
    "lbm_set_stream": [_P, _P],
    "lbm_get_size": [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)],
    "lbm_get_params": [_P, ctypes.POINTER(LbmParams)],
    "lbm_step": [_P, _I],
    "lbm_compute": [_P],
    "lbm_reset": [_P],
    "lbm_update_viscosity": [_P, _F],
    "lbm_set_tau": [_P, _F],
    "lbm_on_click": [_P, _F, _F],
    "lbm_add_obstacle": [_P, _I, _I],
    "lbm_touch_begin": [_P],
    "lbm_touch_move": [_P, _F, _F],
    "lbm_add_external_force": [_P, _F, _F, _F, _F],
    "lbm_build_mask": [ctypes.POINTER(LbmParams), _P],
    "lbm_scene_disks": [ctypes.POINTER(LbmParams), _P, _I, _P],
    "lbm_mask_add_obstacle": [_I, _I, _P, _I, _I],
    "lbm_mask_force_stroke": [_I, _I, _I, _P, _F, _F, _F, _F],
    "lbm_set_info": [_P, _P],
    "lbm_get_info": [_P, _P],
    "lbm_read_macro": [_P, _P, _P, _P],
    "lbm_read_macro_rgba16f": [_P, _P],
    "lbm_read_populations": [_P, _P, _I],
    "lbm_write_populations": [_P, _P, _I],
    "lbm_init_equilibrium": [_P, _P, _P, _P],
    "lbm_conservation": [_P, ctypes.POINTER(_D)],
    "lbm_check_finite": [_P, ctypes.POINTER(ctypes.c_uint64)],
    "lbm_macro_error": [_P, _P, ctypes.POINTER(_D)],
    "lbm_save": [_P, ctypes.c_char_p],
    "lbm_load": [_P, ctypes.c_char_p],
    "lbm_conservation_noalloc": [_P, _I, _I, _P, _I, _I, _P, _P],
    "lbm_apply_edits": [_P, _P, _I, ctypes.POINTER(_I)],
    "lbm_particles_grid": [_I, _I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I)],
    "lbm_particles_init_state": [_P, _I, _I, _P],
    "lbm_particles_create": [_P, _P, ctypes.POINTER(_P)],
    "lbm_particles_destroy": [_P],
    "lbm_particles_info": [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)],
    "lbm_particles_update": [_P, _P],
    "lbm_particles_present": [_P, _P, ctypes.POINTER(_P)],
    "lbm_particles_read": [_P, _P],
    "lbm_particles_write": [_P, _P],
    "lbm_particles_read_canvas": [_P, _P, _P],
    "lbm_particles_counters": [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)],
    "lbm_curl": [_P, _P],
    "lbm_colorize": [_P, _I, _P, _I, _I, _P],
    "lbm_closure_create": [_I, _I, ctypes.c_uint64, ctypes.POINTER(_P)],
    "lbm_closure_destroy": [_P],
    "lbm_closure_set_scales": [_P, _F, _F],
    "lbm_closure_set_form": [_P, _I, _I, _I],
    "lbm_closure_set_kernel": [_P, _I],
    "lbm_closure_set_stress_factor": [_P, _F],
    "lbm_closure_status": [_P],
    "lbm_closure_get_params": [_P, _P],
    "lbm_closure_set_params": [_P, _P],
    "lbm_coarsen": [_P, _P, _I, _F],
    "lbm_closure_apply": [_P, _P],
    "lbm_closure_reserve": [_P, _I, _I, _I],
    "lbm_closure_add_pair": [_P, _P, _P, _I, _I],
    "lbm_closure_pairs": [_P, ctypes.POINTER(_I)],
    "lbm_closure_train": [_P, _I, _F, ctypes.c_uint64, ctypes.POINTER(_D)],
    "lbm_closure_eval": [_P, _I, _I, ctypes.POINTER(_D)],
    "lbm_closure_loss_grad": [_P, _I, _I, _P, _P, ctypes.POINTER(_D), _P],
    "lbm_closure_predict": [_P, _P, _P],
    "lbm_closure_counters": [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)],
    "lbm_status": [_P],
    "lbm_steps_done": [_P, ctypes.POINTER(ctypes.c_uint64)],
    "lbm_kernel_launches": [_P, ctypes.POINTER(ctypes.c_uint64)],
    "lbm_device_macro": [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P)],
    "lbm_device_populations": [_P, ctypes.POINTER(_P), ctypes.POINTER(ctypes.c_int32)],
    "lbm_bounds_report": [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                          ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int32)],
    "lbm_bounds_selftest": [],
    "lbm_batch_generate": [_I, ctypes.c_uint64, _P],
    "lbm_batch_create": [_I, _P, ctypes.POINTER(_P)],
    "lbm_batch_destroy": [_P],
    "lbm_batch_set_stream": [_P, _P],
    "lbm_batch_info": [_P, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_uint64)],
    "lbm_batch_set_config": [_P, _P],
    "lbm_batch_get_config": [_P, _P],
    "lbm_batch_tune": [_P, _I, _P],
    "lbm_batch_step": [_P, _I],
    "lbm_batch_status": [_P],
    "lbm_batch_inject_missing_arrival": [_P, _I, _I, _I, ctypes.c_uint64],
    "lbm_batch_read_macro": [_P, _I, _P, _P, _P],
    "lbm_batch_read_populations": [_P, _I, _P],
    "lbm_batch_read_info": [_P, _I, _P],
    "lbm_batch_conservation": [_P, _I, ctypes.POINTER(_D)],
    "lbm_batch_counters": [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)],
}

_lib = None


def load() -> ctypes.CDLL:
    """Load liblbm.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("liblbm.so is missing at %s: build it with simuverse_gb300.build.build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    lib.lbm_abi_version.restype = ctypes.c_int
    lib.lbm_abi_version.argtypes = []
    lib.lbm_last_error.restype = ctypes.c_char_p
    lib.lbm_last_error.argtypes = []
    lib.lbm_closure_param_count.restype = ctypes.c_int
    lib.lbm_closure_param_count.argtypes = []
    lib.lbm_params_default.restype = None
    lib.lbm_params_default.argtypes = [ctypes.POINTER(LbmParams)]
    lib.lbm_particle_params_default.restype = None
    lib.lbm_particle_params_default.argtypes = [ctypes.POINTER(ParticleParams)]
    for name, args in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = ctypes.c_int
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int) -> int:
    """Raise LbmError for a negative status; return the status otherwise."""
    if code < 0:
        msg = load().lbm_last_error().decode(errors="replace")
        raise LbmError(code, msg)
    return code


def ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def exported_symbols():
    """Names declared in include/lbm.h that the library must export."""
    return ["lbm_abi_version", "lbm_last_error", "lbm_params_default", "lbm_closure_param_count",
            "lbm_particle_params_default"] + list(_SIGNATURES)
