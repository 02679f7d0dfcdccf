"""ctypes binding of the C ABI declared in ``include/pbat_gb300.h``.

The library is the in-tree ``_lib/libpbat_gb300.so``.  It is built on first use when missing (nvcc
is required); there is no fallback implementation: if it cannot be built or loaded, importing the
package's simulation API raises.
"""

from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _build

_lock = threading.Lock()
_lib = None

PBGB_OK = 0
ERRORS = {
    1: "invalid argument",
    2: "CUDA error",
    3: "non-finite state",
    4: "degenerate tetrahedron",
    5: "colour palette overflow",
    6: "no CUDA device",
    7: "device wait timed out",
    8: "internal error",
}


class PbgbError(RuntimeError):
    """A non-zero status returned by the C ABI."""

    def __init__(self, code, message):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}): {message}")
        self.code = code


class VbdDesc(C.Structure):
    """Mirror of ``pbgb_vbd_desc``."""

    _fields_ = [
        ("n_vertices", C.c_int32),
        ("n_tets", C.c_int32),
        ("x", C.c_void_p),
        ("T", C.c_void_p),
        ("v", C.c_void_p),
        ("aext", C.c_void_p),
        ("m", C.c_void_p),
        ("GP", C.c_void_p),
        ("wg", C.c_void_p),
        ("mu", C.c_void_p),
        ("lam", C.c_void_p),
        ("n_partitions", C.c_int32),
        ("Pptr", C.c_void_p),
        ("Padj", C.c_void_p),
        ("init_strategy", C.c_int32),
        ("kD", C.c_double),
        ("detHZero", C.c_double),
        ("acceleration", C.c_int32),
        ("rho", C.c_double),
        ("chebyshev_formula", C.c_int32),
        ("semantics", C.c_int32),
        ("X", C.c_void_p),
        ("n_collision_vertices", C.c_int32),
        ("V", C.c_void_p),
        ("n_collision_triangles", C.c_int32),
        ("F", C.c_void_p),
        ("B", C.c_void_p),
        ("XVA", C.c_void_p),
        ("FA", C.c_void_p),
        ("muC", C.c_double),
        ("muF", C.c_double),
        ("epsv", C.c_double),
        ("active_set_update_frequency", C.c_int32), ("window_size", C.c_int32),
        ("nesterov_lipschitz", C.c_double), ("nesterov_start", C.c_int32),
        ("tr_eta", C.c_double), ("tr_tau", C.c_double), ("tr_curved", C.c_int32),
    ]


# (name, restype, argtypes); every entry point declared in include/pbat_gb300.h.
_vp = C.c_void_p
_i32 = C.c_int32
_f32 = C.c_float
_f64 = C.c_double
_SIGNATURES = [
    ("pbgb_vbd_data_construct", C.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp,
                                         _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("pbgb_vbd_create", C.c_int, [C.POINTER(VbdDesc), C.POINTER(_vp)]),
    ("pbgb_vbd_create_batched", C.c_int, [C.POINTER(VbdDesc), _i32, C.POINTER(_vp)]),
    ("pbgb_vbd_destroy", C.c_int, [_vp]),
    ("pbgb_vbd_step", C.c_int, [_vp, _f32, _i32, _i32]),
    ("pbgb_vbd_synchronize", C.c_int, [_vp]),
    ("pbgb_vbd_get_positions", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_set_positions", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_get_velocities", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_set_velocities", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_set_external_acceleration", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_get_positions_device", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_set_positions_device", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_traced_step", C.c_int, [_vp, _f32, _i32, _i32, _i32, C.c_char_p]),
    ("pbgb_vbd_state_size", C.c_int, [_vp, C.POINTER(C.c_size_t)]),
    ("pbgb_vbd_save_state", C.c_int, [_vp, _vp, C.c_size_t]),
    ("pbgb_vbd_load_state", C.c_int, [_vp, _vp, C.c_size_t]),
    ("pbgb_vbd_trace_next_step", C.c_int, [_vp, C.c_char_p, _i32]),
    ("pbgb_vbd_get_velocities_device", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_set_velocities_device", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_set_material", C.c_int, [_vp, _vp, _vp]),
    ("pbgb_vbd_adjoint_reserve", C.c_int, [_vp, _i32, _i32]),
    ("pbgb_vbd_step_record", C.c_int, [_vp, _f32, _i32, _i32, _i32]),
    ("pbgb_vbd_step_adjoint", C.c_int, [_vp, _i32, _i32, _vp, _vp, _vp, _vp]),
    ("pbgb_vbd_step_adjoint_state", C.c_int, [_vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp]),
    ("pbgb_vbd_get_previous_velocities_device", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_set_previous_velocities_device", C.c_int, [_vp, _vp]),
    ("pbgb_vbd_set_detH_zero", C.c_int, [_vp, _f32]),
    ("pbgb_vbd_set_damping", C.c_int, [_vp, _f32]),
    ("pbgb_vbd_set_strategy", C.c_int, [_vp, _i32]),
    ("pbgb_vbd_set_block_size", C.c_int, [_vp, _i32]),
    ("pbgb_vbd_set_lanes_per_vertex", C.c_int, [_vp, _i32]),
    ("pbgb_vbd_autotune", C.c_int, [_vp, _f32, _i32, _i32, _vp, _vp, _vp]),
    ("pbgb_vbd_set_programmatic_launch", C.c_int, [_vp, _i32]),
    ("pbgb_vbd_set_staged_sweep", C.c_int, [_vp, _i32]),
    ("pbgb_vbd_staged_sweep", C.c_int, [_vp, C.POINTER(_i32), C.POINTER(_i32)]),
    ("pbgb_vbd_set_persistent", C.c_int, [_vp, _i32]),
    ("pbgb_vbd_persistent", C.c_int, [_vp, C.POINTER(_i32)]),
    ("pbgb_vbd_set_batch_tile", C.c_int, [_vp, _i32]),
    ("pbgb_debug_batched_wait", C.c_int, [_vp, C.c_int64, _i32]),
    ("pbgb_vbd_set_scene_bounding_box", C.c_int, [_vp, _vp, _vp]),
    ("pbgb_vbd_sizes", C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    ("pbgb_vbd_launches_per_step", C.c_int, [_vp, _i32, _i32, C.POINTER(C.c_int64)]),
    ("pbgb_vbd_step_graph_kernels", C.c_int, [_vp, C.POINTER(C.c_int64)]),
    ("pbgb_vbd_stream", C.c_int, [_vp, C.POINTER(_vp)]),
    ("pbgb_vbd_set_sweep_timing", C.c_int, [_vp, _i32]),
    ("pbgb_vbd_sweep_timing", C.c_int, [_vp, C.POINTER(_f64), C.POINTER(C.c_int64)]),
    ("pbgb_vbd_get_contacts", C.c_int, [_vp, _vp, _vp]),
    ("pbgb_vbd_get_contact_bvh", C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("pbgb_vbd_objective", C.c_int, [_vp, _f64, C.POINTER(_f64)]),
    ("pbgb_vbd_trust_region_log", C.c_int, [_vp, _vp, _i32, C.POINTER(_i32)]),
    ("pbgb_vbd_gradient", C.c_int, [_vp, _f64, _vp]),
    ("pbgb_vbd_gradient_noalloc", C.c_int, [_vp, _f64, _vp]),
    ("pbgb_last_error", C.c_char_p, [_vp]),
    ("pbgb_debug_adjoint_tet", C.c_int, [_i32, _vp, _vp, _i32, _vp, _vp, _f64, _f64, _vp, _vp, _vp]),
    ("pbgb_bvh_create", C.c_int, [_i32, C.POINTER(_vp)]),
    ("pbgb_bvh_destroy", C.c_int, [_vp]),
    ("pbgb_bvh_build", C.c_int, [_vp, _i32, _vp, _vp, _vp, _vp]),
    ("pbgb_bvh_refit", C.c_int, [_vp, _vp, _vp]),
    ("pbgb_bvh_build_device", C.c_int, [_vp, _i32, _vp, _vp, _vp, _vp]),
    ("pbgb_bvh_stream", C.c_int, [_vp, C.POINTER(_vp)]),
    ("pbgb_bvh_topology", C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("pbgb_bvh_overlaps", C.c_int, [_vp, _i32, _vp, _vp, _vp, C.c_int64, C.POINTER(C.c_int64)]),
    ("pbgb_bvh_self_overlaps", C.c_int, [_vp, _vp, _vp, C.c_int64, C.POINTER(C.c_int64)]),
    ("pbgb_bvh_nearest_simplices", C.c_int, [_vp, _i32, _vp, _i32, _vp, _i32, _vp, _i32, _vp]),
    ("pbgb_bvh_visits", C.c_int, [_vp, _vp]),
    ("pbgb_simplex_boxes", C.c_int, [_i32, _vp, _i32, _vp, _i32, _vp, _vp]),
    ("pbgb_bvh_last_error", C.c_char_p, [_vp]),
    ("pbgb_ccd_create", C.c_int, [_i32, _i32, _vp, _i32, _vp, _vp, C.POINTER(_vp)]),
    ("pbgb_ccd_destroy", C.c_int, [_vp]),
    ("pbgb_ccd_initialize", C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    ("pbgb_ccd_update", C.c_int, [_vp, _vp]),
    ("pbgb_ccd_finalize", C.c_int, [_vp, _vp]),
    ("pbgb_ccd_get", C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    ("pbgb_ccd_last_error", C.c_char_p, [_vp]),
    ("pbgb_debug_vertex_triangle_contact", C.c_int, [_vp, _vp, _vp, _vp, _f32, _f32, _f32, _f32, _vp, _vp, _vp]),
    ("pbgb_debug_vertex_block", C.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _f64, _f64,
                                         _f64, _f64, _f64, _vp, _vp, _vp]),
]

SYMBOLS = [s[0] for s in _SIGNATURES]


def lib():
    """Load (building first if needed) the CUDA library."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            L = C.CDLL(str(path))
            for name, res, args in _SIGNATURES:
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(rc, handle=None):
    if rc != PBGB_OK:
        msg = lib().pbgb_last_error(handle)
        raise PbgbError(rc, msg.decode() if msg else "")


def check_ccd(rc, ccd=None):
    if rc != PBGB_OK:
        msg = lib().pbgb_ccd_last_error(ccd)
        raise PbgbError(rc, msg.decode() if msg else "")


def check_bvh(rc, bvh=None):
    if rc != PBGB_OK:
        msg = lib().pbgb_bvh_last_error(bvh)
        raise PbgbError(rc, msg.decode() if msg else "")


def ptr(a):
    """Raw data pointer of a contiguous numpy array (None -> NULL)."""
    if a is None:
        return None
    return a.ctypes.data


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)
