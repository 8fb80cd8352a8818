"""ctypes binding of the C ABI in include/jitter_gpu.h.

The plain structs are mirrored twice: as numpy structured dtypes (bulk upload of whole
scenes) and as ctypes structures (single records).  The library is loaded from the
package directory; if it is missing the import fails loudly — there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libjitter_gpu.so")

JG_OK = 0
JG_ERR_INVALID_ARG = -1
JG_ERR_CAPACITY = -2
JG_ERR_NONFINITE = -3
JG_ERR_TIMEOUT = -4
JG_ERR_CUDA = -5
JG_ERR_NOT_SUPPORTED = -6
JG_ERR_INVALID_SHAPE = -7

MOTION_DYNAMIC, MOTION_KINEMATIC, MOTION_STATIC = 0, 1, 2
SHAPE_BOX, SHAPE_SPHERE, SHAPE_CAPSULE, SHAPE_CYLINDER, SHAPE_CONE, SHAPE_POINTCLOUD, SHAPE_TRIANGLE = range(7)
BODY_ACTIVE = 1 << 2
BODY_GYROSCOPIC = 1 << 3
BODY_LOCKS_SHIFT = 4
BODY_NO_GRAVITY = 1 << 12
BODY_SPECULATIVE = 1 << 13   # RigidBody.EnableSpeculativeContacts
RESID_MAX = 2048                # iterations whose residual a step records (jg_get_residuals)
COLLIDE_NOALLOC_MAX_PAIRS = 16384  # JG_COLLIDE_NOALLOC_MAX_PAIRS
MLP_IN, MLP_HID, MLP_OUT = 24, 64, 3
MLP_NW = MLP_HID * MLP_IN + MLP_HID + MLP_HID * MLP_HID + MLP_HID + MLP_OUT * MLP_HID + MLP_OUT  # trainable
MLP_NPARAM = MLP_NW + MLP_IN + MLP_IN + MLP_OUT  # + feature mean, feature scale, output scale
WARMSTART_ZERO, WARMSTART_CACHED, WARMSTART_MLP = 0, 1, 2
CONSTRAINT_BALLSOCKET, CONSTRAINT_HINGEANGLE, CONSTRAINT_DISTANCELIMIT, CONSTRAINT_CONELIMIT, CONSTRAINT_TWISTANGLE = 1, 2, 3, 4, 5
CONSTRAINT_FIXEDANGLE, CONSTRAINT_POINTONPLANE, CONSTRAINT_ANGULARMOTOR, CONSTRAINT_LINEARMOTOR = 6, 7, 8, 9
CONSTRAINT_ANGULARSERVO, CONSTRAINT_LINEARSERVO, CONSTRAINT_LINEARAXISSERVO, CONSTRAINT_TWISTSERVO = 10, 11, 12, 13
CONSTRAINT_POINTONLINE, CONSTRAINT_ELLIPTICALCONELIMIT = 14, 15

ERROR_NAMES = {
    JG_ERR_INVALID_ARG: "JG_ERR_INVALID_ARG", JG_ERR_CAPACITY: "JG_ERR_CAPACITY",
    JG_ERR_NONFINITE: "JG_ERR_NONFINITE", JG_ERR_TIMEOUT: "JG_ERR_TIMEOUT", JG_ERR_CUDA: "JG_ERR_CUDA",
    JG_ERR_NOT_SUPPORTED: "JG_ERR_NOT_SUPPORTED", JG_ERR_INVALID_SHAPE: "JG_ERR_INVALID_SHAPE",
}

PARAMS_FIELDS = [
    ("gravity", ctypes.c_float * 3), ("substeps", ctypes.c_int32), ("solver_iterations", ctypes.c_int32),
    ("relax_iterations", ctypes.c_int32), ("enable_auxiliary_contacts", ctypes.c_int32),
    ("persistent_manifold", ctypes.c_int32), ("speculative_relaxation", ctypes.c_float),
    ("edge_filter", ctypes.c_int32), ("warm_start_mode", ctypes.c_int32), ("max_bodies", ctypes.c_int32),
    ("max_shapes", ctypes.c_int32), ("max_pairs", ctypes.c_int32), ("max_arbiters", ctypes.c_int32),
    ("max_constraints", ctypes.c_int32), ("solver_block", ctypes.c_int32), ("solver_ctas_per_sm", ctypes.c_int32),
    ("narrow_tile", ctypes.c_int32), ("use_graph", ctypes.c_int32), ("record_residual", ctypes.c_int32),
    ("deterministic", ctypes.c_int32),
    ("partitioned_solve", ctypes.c_int32), ("speculative_threshold", ctypes.c_float),
    ("allow_deactivation", ctypes.c_int32),
    ("sched_cells_per_sm", ctypes.c_float),
]


class WorldParams(ctypes.Structure):
    _fields_ = PARAMS_FIELDS


BODY_DTYPE = np.dtype([
    ("position", "<f4", 3), ("orientation", "<f4", 4), ("velocity", "<f4", 3), ("angular_velocity", "<f4", 3),
    ("delta_velocity", "<f4", 3), ("delta_angular_velocity", "<f4", 3), ("inv_inertia", "<f4", 6),
    ("inv_mass", "<f4"), ("friction", "<f4"), ("restitution", "<f4"), ("linear_damping", "<f4"),
    ("angular_damping", "<f4"), ("force", "<f4", 3), ("torque", "<f4", 3), ("motion_type", "<i4"),
    ("flags", "<i4"), ("world", "<i4"),
])
SHAPE_DTYPE = np.dtype([
    ("kind", "<i4"), ("body", "<i4"), ("dims", "<f4", 4), ("center", "<f4", 3), ("data_offset", "<i4"),
    ("data_count", "<i4"),
])
TRIANGLE_DTYPE = np.dtype([
    ("a", "<f4", 3), ("b", "<f4", 3), ("c", "<f4", 3), ("normal", "<f4", 3), ("neighbor", "<i4", 3), ("pad", "<i4"),
])
CONTACT_DTYPE = np.dtype([
    ("shape1", "<i4"), ("shape2", "<i4"), ("body1", "<i4"), ("body2", "<i4"), ("slot", "<i4"),
    ("usage_mask", "<i4"), ("color", "<i4"), ("flags", "<i4"), ("normal", "<f4", 3), ("tangent1", "<f4", 3),
    ("tangent2", "<f4", 3), ("rel_pos1", "<f4", 3), ("rel_pos2", "<f4", 3), ("pos1_local", "<f4", 3),
    ("pos2_local", "<f4", 3), ("accumulated", "<f4", 3), ("mass", "<f4", 3), ("bias", "<f4"),
    ("penalty_bias", "<f4"), ("friction", "<f4"), ("restitution", "<f4"),
])
COUNTER_NAMES = ["pairs", "colliding", "manifold_points", "arbiters", "contacts", "new_contacts", "colors",
                 "epa_calls", "epa_failures", "exact_fallbacks", "status", "created_arbiters", "removed_arbiters",
                 "kernel_launches", "solver_tasks", "task_arbiters", "task_colors", "speculative_contacts"]
TIMING_NAMES = ["broadphase", "narrowphase", "add_arbiter", "coloring", "solve", "update_contacts",
                "update_bodies", "total"]

# every entry point declared by include/jitter_gpu.h: name -> (restype, argtypes)
_P = ctypes.c_void_p
_I = ctypes.c_int32
_F = ctypes.c_float
_PF = ctypes.POINTER(ctypes.c_float)
_PI = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.c_int64
SIGNATURES = {
    "jg_default_params": (_I, [_P]),
    "jg_create": (_I, [_P, ctypes.POINTER(_P)]),
    "jg_destroy": (_I, [_P]),
    "jg_set_params": (_I, [_P, _P]),
    "jg_get_params": (_I, [_P, _P]),
    "jg_upload_bodies": (_I, [_P, _P, _I]),
    "jg_download_bodies": (_I, [_P, _P, _I]),
    "jg_upload_shapes": (_I, [_P, _P, _I, _P, _I, _P, _I]),
    "jg_set_body": (_I, [_P, _I, _I, _P]),
    "jg_activate_body": (_I, [_P, _I]),
    "jg_set_body_sleep": (_I, [_P, _I, _F, _F, _F]),
    "jg_add_constraint": (_I, [_P, _I, _I, _I, _P, _PI]),
    "jg_set_servo": (_I, [_P, _I, _P, ctypes.c_float]),
    "jg_set_constraint_params": (_I, [_P, _I, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
    "jg_step": (_I, [_P, _F]),
    "jg_step_host": (_I, [_P, _F, _P, _I]),
    "jg_stabilize": (_I, [_P, _F, _I, _I]),
    "jg_collide_pairs": (_I, [_P, _P, _I, _P, _P]),
    "jg_collide_pairs_noalloc": (_I, [_P, _P, _I, _P, _P]),
    "jg_manifold_pairs": (_I, [_P, _P, _I, _P, _P, _P]),
    "jg_get_pairs": (_I, [_P, _P, _I, _PI]),
    "jg_get_contacts": (_I, [_P, _P, _I, _PI]),
    "jg_get_arbiter_events": (_I, [_P, _P, _I, _PI, _P, _I, _PI]),
    "jg_get_constraints": (_I, [_P, _P, _P, _I, _PI]),
    "jg_get_counters": (_I, [_P, _P]),
    "jg_get_timings": (_I, [_P, _P]),
    "jg_get_residuals": (_I, [_P, _P, _I, _PI]),
    "jg_export_state": (_I, [_P, _P, _I64, ctypes.POINTER(_I64)]),
    "jg_import_state": (_I, [_P, _P, _I64]),
    "jg_check_state": (_I, [_P, _I64, _I, _I, _I, _I]),
    "jg_mlp_load": (_I, [_P, _P, _I]),
    "jg_mlp_predict": (_I, [_P, _P, _I, _P]),
    "jg_mlp_train_step": (_I, [_P, _P, _P, _I, _F, _PF]),
    "jg_mlp_export": (_I, [_P, _P, _I, _PI]),
    "jg_mlp_gradients": (_I, [_P, _P, _P, _I, _P, _I, _PF]),
    "jg_collect_training": (_I, [_P, _P, _P, _I, _PI]),
    "jg_batch_create": (_I, [_P, _I, ctypes.POINTER(_P)]),
    "jg_batch_step": (_I, [_P, _F]),
    "jg_autotune": (_I, [_P, _F, _I, _P]),
    "jg_shape_mass_inertia": (_I, [_P, _P, _P, _P, _P]),
    "jg_last_error": (ctypes.c_char_p, []),
    "jg_version": (ctypes.c_char_p, []),
}

_lib = None


def load(path=LIB_PATH):
    """Loads libjitter_gpu.so and declares every entry point; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libjitter_gpu.so not built (run jitterphysics2_gb300.build.build()); "
                          "the library has no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class JitterError(RuntimeError):
    def __init__(self, code, what=""):
        lib = _lib
        msg = lib.jg_last_error().decode() if lib is not None else ""
        super().__init__("%s failed: %s (%d) %s" % (what, ERROR_NAMES.get(code, "?"), code, msg))
        self.code = code


def check(code, what=""):
    if code != JG_OK:
        raise JitterError(code, what)
    return code


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else None


# The values jg_default_params writes (a freshly constructed World, World.cs:333-416,
# World.Detect.cs:88-122), for callers that fill a jg_world_params without loading the
# library (the CPU oracle and the reference arm of the benchmark).
PARAM_DEFAULTS = dict(gravity=(0.0, -9.81, 0.0), substeps=1, solver_iterations=6, relax_iterations=4,
                      enable_auxiliary_contacts=1, persistent_manifold=1, speculative_relaxation=0.9,
                      speculative_threshold=10.0, edge_filter=1, warm_start_mode=1, narrow_tile=32, allow_deactivation=1,
                      partitioned_solve=1)


def params_struct(**kw):
    """A jg_world_params with the defaults of jg_default_params and the given fields,
    built without loading libjitter_gpu.so."""
    p = WorldParams()
    for k, v in dict(PARAM_DEFAULTS, **kw).items():
        if k == "gravity":
            p.gravity[0], p.gravity[1], p.gravity[2] = v
        else:
            setattr(p, k, v)
    return p


def default_params(**kw):
    p = WorldParams()
    load().jg_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if k == "gravity":
            p.gravity[0], p.gravity[1], p.gravity[2] = v
        else:
            setattr(p, k, v)
    return p


def mass_inertia(shape_row, hull=None):
    """(inertia6, com3, mass) of one SHAPE_DTYPE record, CalculateMassInertia of its shape."""
    lib = load()
    rec = np.array([shape_row], dtype=SHAPE_DTYPE) if not isinstance(shape_row, np.ndarray) else shape_row.reshape(1)
    I6 = np.zeros(6, np.float32)
    com = np.zeros(3, np.float32)
    m = np.zeros(1, np.float32)
    h = np.ascontiguousarray(hull, np.float32) if hull is not None else None
    check(lib.jg_shape_mass_inertia(ptr(rec), ptr(h), ptr(I6), ptr(com), ptr(m)), "jg_shape_mass_inertia")
    return I6, com, float(m[0])
