"""ctypes mirror of include/gbmpm.h and the loader of the native library.

The native library (libgbmpm.so, built in-tree by mpm_engine_gb300.build) is the
only compute path. Loading fails loudly when it has not been built; there is no
Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

MAX_MATERIALS = 16
MAX_COLLIDERS = 32
NUM_PHASES = 6

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_STATE = 3
ERR_BOUNDS = 4
ERR_UNSUPPORTED = 5

FLAG_STENCIL_OOB = 1
FLAG_NONFINITE = 2
FLAG_LIST_OVERFLOW = 4

TICK_FUSED = 1
TICK_GRAPH = 2
TICK_PROFILE = 4
TICK_REORDER = 8
TICK_DETERMINISTIC = 16
# gbmpm_set_resort's automatic setting: ticks of S >= 100 substeps in scenes of 150,000
# particles or more re-sort every max(50, S / 3) substeps
RESORT_AUTO = -1

COLLIDER_PLANE = 0
COLLIDER_BOX = 1
COLLIDER_CUP = 2
COLLIDER_WALLS = 3
COLLIDER_SDF = 4

_F16 = C.c_float * MAX_MATERIALS


class Particles(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("x", C.c_void_p), ("v", C.c_void_p),
        ("C", C.c_void_p), ("F", C.c_void_p), ("F_trial", C.c_void_p), ("L", C.c_void_p),
        ("stress", C.c_void_p),
        ("mass", C.c_void_p), ("vol", C.c_void_p), ("density", C.c_void_p), ("Jp", C.c_void_p),
        ("mu", C.c_void_p), ("lam", C.c_void_p), ("yield_stress", C.c_void_p),
        ("material", C.c_void_p), ("selection", C.c_void_p),
        ("cov", C.c_void_p), ("init_cov", C.c_void_p),
        ("cdf_tag", C.c_void_p),
        ("rigid_id", C.c_void_p), ("x_ref", C.c_void_p), ("mod_mask", C.c_void_p),
    ]


class Grid(C.Structure):
    _fields_ = [("n_grid", C.c_int32), ("mv", C.c_void_p), ("v", C.c_void_p)]


class Model(C.Structure):
    _fields_ = [
        ("n_grid", C.c_int32),
        ("grid_lim", C.c_float), ("dx", C.c_float), ("inv_dx", C.c_float),
        ("gravity", C.c_float * 3),
        ("rpic_damping", C.c_float), ("grid_v_damping_scale", C.c_float),
        ("periodic_x", C.c_int32), ("update_cov_with_F", C.c_int32),
        ("material_mask", C.c_uint32),
        ("E", _F16), ("nu", _F16), ("bulk", _F16), ("hardening", _F16), ("xi", _F16),
        ("plastic_viscosity", _F16), ("softening", _F16), ("alpha", _F16),
        ("muI_mu_s", _F16), ("muI_delta_mu", _F16), ("muI_I0", _F16), ("muI_d", _F16),
        ("muI_rho_s", _F16), ("muI_phi_init", _F16), ("muI_phi_chi", _F16),
        ("eta_table", C.c_void_p), ("eta_table_n", C.c_int32),
        ("eta_table_smin", C.c_float), ("eta_table_smax", C.c_float),
    ]


class Collider(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("surface_type", C.c_int32), ("reset", C.c_int32), ("sdf_res", C.c_int32),
        ("start_time", C.c_float), ("end_time", C.c_float),
        ("point", C.c_float * 3), ("normal", C.c_float * 3), ("size", C.c_float * 3),
        ("velocity", C.c_float * 3), ("omega", C.c_float * 3),
        ("rot", C.c_float * 9), ("quat", C.c_float * 4),
        ("friction", C.c_float),
        ("outer_radius", C.c_float), ("inner_radius", C.c_float), ("half_height", C.c_float),
        ("inner_floor_z", C.c_float), ("fillet_radius", C.c_float),
        ("sticky_depth", C.c_float), ("contact_band", C.c_float),
        ("sdf_origin", C.c_float * 3), ("sdf_cell", C.c_float), ("band", C.c_float),
        ("sdf_val", C.c_void_p), ("sdf_grad", C.c_void_p),
        ("rot64", C.c_double * 9),
    ]


MAX_CDF = 4


class Cdf(C.Structure):
    _fields_ = [
        ("values", C.c_void_p), ("valid", C.c_void_p), ("res", C.c_int32), ("surface_type", C.c_int32),
        ("origin", C.c_float * 3), ("cell", C.c_float), ("center", C.c_float * 3), ("quat", C.c_float * 4),
        ("velocity", C.c_float * 3), ("omega", C.c_float * 3), ("band", C.c_float), ("friction", C.c_float),
        ("start_time", C.c_float), ("end_time", C.c_float),
    ]


class RigidBody(C.Structure):
    """gbmpm_rigid_body: R and the body-frame inverse inertia row-major."""
    _fields_ = [("x_cm", C.c_float * 3), ("v_cm", C.c_float * 3), ("omega", C.c_float * 3), ("R", C.c_float * 9),
                ("mass", C.c_float), ("inv_inertia", C.c_float * 9)]


class RigidSurface(C.Structure):
    _fields_ = [("point", C.c_double * 3), ("normal", C.c_double * 3), ("friction", C.c_double),
                ("restitution", C.c_double), ("start_time", C.c_double), ("end_time", C.c_double)]


class Modifier(C.Structure):
    """gbmpm_modifier: kind 0 impulse, 1 velocity translation, 2 velocity rotation."""
    _fields_ = [("kind", C.c_int32), ("start_time", C.c_float), ("end_time", C.c_float), ("vec", C.c_float * 3),
                ("point", C.c_float * 3), ("normal", C.c_float * 3), ("axis1", C.c_float * 3),
                ("axis2", C.c_float * 3), ("rotation_scale", C.c_float), ("translation_scale", C.c_float)]


MAX_RIGID_SURFACES = 8
MAX_MODIFIERS = 32


class AdjGrads(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("x", "v", "C", "F_trial", "yield_stress", "mu", "lam", "L", "viscosity",
                                          "Jp", "collider_force", "collider_velocity")]


class FieldPoints(C.Structure):
    """gbmpm_field_points: explicit device points, or the res^3 grid (points = None)."""
    _fields_ = [("points", C.c_void_p), ("n", C.c_int64), ("origin", C.c_double * 3), ("cell", C.c_double),
                ("res", C.c_int32)]


# every entry point include/gbmpm.h declares, with its ctypes signature
_SIGNATURES = {
    "gbmpm_last_error": (C.c_char_p, []),
    "gbmpm_phase_name": (C.c_char_p, [C.c_int32]),
    "gbmpm_engine_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "gbmpm_engine_destroy": (None, [C.c_void_p]),
    "gbmpm_bind": (C.c_int, [C.c_void_p, C.POINTER(Particles), C.POINTER(Grid)]),
    "gbmpm_set_model": (C.c_int, [C.c_void_p, C.POINTER(Model)]),
    "gbmpm_set_colliders": (C.c_int, [C.c_void_p, C.POINTER(Collider), C.c_int32]),
    "gbmpm_get_colliders": (C.c_int, [C.c_void_p, C.POINTER(Collider), C.c_int32]),
    "gbmpm_tick": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_int32, C.c_int32,
                             C.c_void_p]),
    "gbmpm_guard": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.c_void_p]),
    "gbmpm_wrench": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_void_p]),
    "gbmpm_reset_wrench": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gbmpm_set_cdf": (C.c_int, [C.c_void_p, C.POINTER(Cdf), C.c_int32]),
    "gbmpm_get_cdf": (C.c_int, [C.c_void_p, C.POINTER(Cdf), C.c_int32]),
    "gbmpm_cdf_wrench": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_void_p]),
    "gbmpm_reset_cdf_wrench": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gbmpm_cdf_grids": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64), C.c_void_p]),
    "gbmpm_compute_cauchy": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                       C.POINTER(C.c_int32), C.c_void_p]),
    "gbmpm_contact_wrench": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double,
                                       C.c_int32, C.c_int32, C.POINTER(C.c_double), C.c_void_p]),
    "gbmpm_adjoint_segment": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_int32,
                                        C.POINTER(AdjGrads), C.c_void_p]),
    "gbmpm_adjoint_forward": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_int32, C.c_void_p,
                                        C.c_void_p]),
    "gbmpm_adjoint_reverse": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_int32, C.c_void_p,
                                        C.POINTER(AdjGrads), C.c_void_p]),
    "gbmpm_sort_particles": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(C.c_int32), C.c_void_p,
                                       C.c_void_p]),
    "gbmpm_rebuild_active_blocks": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_void_p]),
    "gbmpm_compute_R": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gbmpm_compute_cov": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gbmpm_profile": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_int32]),
    "gbmpm_guard_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_float),
                                      C.POINTER(C.c_int32), C.c_void_p]),
    "gbmpm_launch_count": (C.c_int64, [C.c_void_p]),
    "gbmpm_set_tuning": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "gbmpm_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "gbmpm_set_resort": (C.c_int, [C.c_void_p, C.c_int32]),
    "gbmpm_get_resort": (C.c_int32, [C.c_void_p]),
    "gbmpm_debug_deposit_sums": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(C.c_double), C.c_void_p]),
    "gbmpm_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]),
    "gbmpm_batch_destroy": (None, [C.c_void_p]),
    "gbmpm_batch_tick": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_int32, C.c_int32,
                                   C.c_void_p]),
    "gbmpm_batch_guard": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.c_void_p]),
    "gbmpm_batch_launch_count": (C.c_int64, [C.c_void_p]),
    "gbmpm_batch_set_tuning": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "gbmpm_batch_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "gbmpm_cdf_restamp": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p]),
    "gbmpm_cdf_force_stamp": (C.c_int, [C.c_void_p, C.c_int32]),
    "gbmpm_cdf_mask_off": (C.c_int, [C.c_void_p, C.c_int32]),
    "gbmpm_graph_state": (C.c_int32, [C.c_void_p]),
    "gbmpm_debug_fail_next_capture": (C.c_int, [C.c_void_p]),
    "gbmpm_batch_graph_state": (C.c_int32, [C.c_void_p]),
    "gbmpm_batch_debug_fail_next_capture": (C.c_int, [C.c_void_p]),
    "gbmpm_set_rigid": (C.c_int, [C.c_void_p, C.POINTER(RigidBody), C.c_int32, C.POINTER(RigidSurface), C.c_int32]),
    "gbmpm_get_rigid": (C.c_int, [C.c_void_p, C.POINTER(RigidBody), C.c_int32, C.c_void_p]),
    "gbmpm_set_modifiers": (C.c_int, [C.c_void_p, C.POINTER(Modifier), C.c_int32]),
    "gbmpm_field_nearest": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gbmpm_field_winding": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p]),
    "gbmpm_field_tri_distance": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
}

PACKAGE_DIR = Path(__file__).resolve().parent
LIB_PATH = PACKAGE_DIR / "_build" / "libgbmpm.so"

_lib = None


class NativeError(RuntimeError):
    pass


def library_path() -> Path:
    return Path(os.environ.get("GBMPM_LIBRARY", str(LIB_PATH)))


def load() -> C.CDLL:
    """Load libgbmpm.so and bind every declared entry point (raises if missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise NativeError(
            f"native library {path} not found: build it with "
            f"`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
    lib = C.CDLL(str(path))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def declared_symbols() -> list[str]:
    return list(_SIGNATURES)


def check(rc: int, what: str = "") -> None:
    """Map a gbmpm_status to the reference's exception types."""
    if rc == OK:
        return
    msg = (_lib.gbmpm_last_error() or b"").decode() if _lib is not None else ""
    text = f"{what}: {msg}" if what else msg
    if rc == ERR_ARG:
        raise ValueError(text)
    if rc == ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    raise NativeError(f"{text} (status {rc})")
