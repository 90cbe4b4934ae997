"""ctypes view of the C ABI in include/hbtu.h (libhbtu.so).

The structures below mirror include/hbtu.h field by field.  ``load()`` never
falls back to anything: if the CUDA library is missing it raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

HBTU_OK = 0
HBTU_ERR_INVALID_ARGUMENT = 1
HBTU_ERR_CUDA = 2
HBTU_ERR_OUT_OF_MEMORY = 3
HBTU_ERR_NOT_CONVERGED = 4
HBTU_ERR_NO_DEVICE = 5
HBTU_ERR_TOO_LARGE = 6

HBTU_NOALLOC_MAX_PARTICLES = 16384

HBTU_PRECISION_FP32 = 0
HBTU_PRECISION_FP64 = 1
HBTU_HOST = 0
HBTU_DEVICE = 1

STATUS_NAMES = {0: "HBTU_OK", 1: "HBTU_ERR_INVALID_ARGUMENT", 2: "HBTU_ERR_CUDA",
                3: "HBTU_ERR_OUT_OF_MEMORY", 4: "HBTU_ERR_NOT_CONVERGED",
                5: "HBTU_ERR_NO_DEVICE", 6: "HBTU_ERR_TOO_LARGE"}


class hbtu_params(C.Structure):
    _fields_ = [
        ("softening", C.c_double), ("open_angle", C.c_double),
        ("bound_mass_precision", C.c_double), ("min_num_part", C.c_int64),
        ("max_sample_size", C.c_int64), ("refine_mostbound", C.c_int32),
        ("periodic", C.c_int32), ("box_size", C.c_double), ("G", C.c_double),
        ("hubble", C.c_double), ("scale_factor", C.c_double), ("precision", C.c_int32),
        ("max_passes", C.c_int32), ("device", C.c_int32), ("reserved", C.c_int32),
    ]


class hbtu_state(C.Structure):
    _fields_ = [
        ("ref_pos", C.c_float * 3), ("ref_vel", C.c_float * 3),
        ("mostbound_pos", C.c_float * 3), ("mostbound_vel", C.c_float * 3),
        ("mostbound_id", C.c_int64),
    ]


class hbtu_result(C.Structure):
    _fields_ = [
        ("nbound", C.c_int64), ("mbound", C.c_float),
        ("ref_pos", C.c_float * 3), ("ref_vel", C.c_float * 3),
        ("mostbound_pos", C.c_float * 3), ("mostbound_vel", C.c_float * 3),
        ("specific_potential", C.c_float), ("specific_kinetic", C.c_float),
        ("specific_angmom", C.c_float * 3), ("nbound_type", C.c_int64 * 6),
        ("mbound_type", C.c_float * 6), ("iterations", C.c_int32),
        ("disrupted", C.c_int32), ("converged", C.c_int32), ("too_few", C.c_int32),
        ("evaluations", C.c_int64), ("interactions", C.c_int64), ("status", C.c_int32),
        ("reserved", C.c_int32),
    ]


class hbtu_particles(C.Structure):
    _fields_ = [
        ("id", C.c_void_p), ("pos", C.c_void_p), ("vel", C.c_void_p), ("mass", C.c_void_p),
        ("type", C.c_void_p), ("location", C.c_int32), ("reserved", C.c_int32),
    ]


class hbtu_props(C.Structure):
    _fields_ = [
        ("rmax_comoving", C.c_float), ("vmax_physical", C.c_float),
        ("last_max_vmax_physical", C.c_float), ("snapshot_of_last_max_vmax", C.c_int32),
        ("r2sigma_comoving", C.c_float), ("rhalf_comoving", C.c_float),
        ("r200crit_comoving", C.c_float), ("m200crit", C.c_float),
        ("inertial_tensor", C.c_float * 6), ("inertial_tensor_weighted", C.c_float * 6),
    ]


class hbtu_core(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("sigma_r", C.c_float), ("vel", C.c_float * 3),
                ("sigma_v", C.c_float)]


class hbtu_stats(C.Structure):
    _fields_ = [
        ("total_ms", C.c_double), ("tree_ms", C.c_double), ("walk_ms", C.c_double),
        ("loop_ms", C.c_double), ("calls", C.c_int64), ("passes", C.c_int64),
        ("kernel_launches", C.c_int64), ("walk_launches", C.c_int64),
        ("evaluations", C.c_int64), ("interactions", C.c_int64),
        ("walk1_ms", C.c_double), ("walk1_interactions", C.c_int64),
        ("small_ms", C.c_double), ("small_subhaloes", C.c_int64),
    ]


# every entry point declared in include/hbtu.h: name -> (restype, argtypes)
SIGNATURES = {
    "hbtu_create": (C.c_int, [C.POINTER(hbtu_params), C.POINTER(C.c_void_p)]),
    "hbtu_destroy": (C.c_int, [C.c_void_p]),
    "hbtu_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hbtu_unbind": (C.c_int, [C.c_void_p, C.POINTER(hbtu_particles), C.c_int64,
                              C.POINTER(hbtu_state), C.c_void_p, C.c_void_p, C.c_void_p]),
    "hbtu_unbind_batch": (C.c_int, [C.c_void_p, C.POINTER(hbtu_particles), C.c_int64,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p]),
    "hbtu_binding_energies": (C.c_int, [C.c_void_p, C.POINTER(hbtu_particles), C.c_int64,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "hbtu_last_error": (C.c_char_p, [C.c_void_p]),
    "hbtu_direct_potential": (C.c_int, [C.c_void_p, C.POINTER(hbtu_particles), C.c_int64,
                                        C.c_void_p, C.c_int64, C.c_void_p]),
    "hbtu_energy_gradient": (C.c_int, [C.c_void_p, C.POINTER(hbtu_particles), C.c_int64,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]),
    "hbtu_set_timing": (C.c_int, [C.c_void_p, C.c_int32]),
    "hbtu_set_option": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
    "hbtu_get_option": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int64)]),
    "hbtu_get_stats": (C.c_int, [C.c_void_p, C.POINTER(hbtu_stats)]),
    "hbtu_reset_stats": (C.c_int, [C.c_void_p]),
    "hbtu_version": (C.c_int32, []),
    "hbtu_unbind_noalloc": (C.c_int, [C.POINTER(hbtu_params), C.POINTER(hbtu_particles), C.c_int64,
                                      C.POINTER(hbtu_state), C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]),
    "hbtu_subhalo_properties": (C.c_int, [C.c_void_p, C.POINTER(hbtu_particles), C.c_int64,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_int32, C.c_void_p]),
    "hbtu_merge_detect": (C.c_int, [C.c_void_p, C.POINTER(hbtu_particles), C.c_int64,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "hbtu_index_create": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "hbtu_index_destroy": (C.c_int, [C.c_void_p]),
    "hbtu_index_fill": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                  C.c_int32]),
    "hbtu_index_lookup": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32]),
    "hbtu_index_key_range": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
}

_LIB = None


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libhbtu.so (building it first if needed and possible)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"CUDA library not built: {path}")
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class HBTUError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def check(status: int, handle=None) -> None:
    if status != HBTU_OK:
        lib = load()
        msg = lib.hbtu_last_error(handle)
        raise HBTUError(status, msg.decode() if msg else "")
