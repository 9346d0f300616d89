"""ctypes binding of include/dio_cuda.h.

numpy structured dtypes mirror the C records (and thereby the reference's
#[repr(C)] structs) byte for byte; `lib()` loads the in-tree
libdio_cuda.so and raises if it is missing -- there is no fallback path.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdio_cuda.so")

# ---------------------------------------------------------------- status
DIO_OK = 0
DIO_ERR_INVALID = 1
DIO_ERR_CAPACITY = 2
DIO_ERR_TIMEOUT = 3
DIO_ERR_CUDA = 4
DIO_ERR_NONFINITE = 5
DIO_ERR_STATE = 6

SPHERE, CUBE, TETRAHEDRON, BOX, HULL = 0, 1, 2, 3, 4
CONTAINER = 0xFFFFFFFF
SPRING, ROD, BALL_SOCKET, ROPE = 0, 1, 2, 3
CONTACTS_PER_PAIR = 4
# header of a dio_world_checkpoint image (16-byte aligned sections follow:
# bodies, state, joints, scene table, hull vertices, poses / velocities in
# the world's precision, the last step's rows, the last step's narrow slots
# of a contact-lag world)
CKPT_HEADER = np.dtype([("magic", "S8"), ("version", "<u4"), ("precision", "<u4"), ("p_bytes", "<u4"),
                        ("r_bytes", "<u4"), ("n", "<u4"), ("n_joints", "<u4"), ("n_scenes", "<u4"),
                        ("n_hull", "<u4"), ("rows", "<u4"), ("pair_rows", "<u4"), ("has_container", "<u4"),
                        ("per_pair", "<u4"), ("lag_pairs", "<u4"), ("pad", "<u4"), ("steps", "<u8"),
                        ("total_bytes", "<u8")])
PRIMAL_VARIANTS = 11  # DIO_PRIMAL_VARIANTS
XFORM_POSE, XFORM_MAT4 = 0, 1  # DIO_XFORM_*
DEBUG_EPA_NO_FIRST_WAIT = 1  # DIO_DEBUG_EPA_NO_FIRST_WAIT (DioConfig.debug_flags, tests only)
SOLVE_AUTO, SOLVE_PER_PHASE = 0, 1  # DioSolveLaunch (DioConfig.batched_solver)

SOLVER_JACOBI, SOLVER_COLORED = 0, 1
PREC_F32, PREC_SPLIT, PREC_F64 = 0, 1, 2

# ------------------------------------------------------------ record dtypes
SHAPE = np.dtype([("tag", "<u4"), ("pad", "<u4", 3), ("corners", "<f4", (4, 4))])
BODY = np.dtype([("position", "<f4", 4), ("orientation", "<f4", 4), ("shape", SHAPE)])
# DioBodyMotion: the per-frame pose and velocities of a body (64 B)
MOTION = np.dtype([("position", "<f4", 3), ("orientation", "<f4", 4), ("velocity", "<f4", 3),
                   ("angular_velocity", "<f4", 3), ("prev_velocity", "<f4", 3)])
PAIR = np.dtype([("a", "<u4"), ("b", "<u4")])
CONTACT_OUT = np.dtype([("valid", "<u4"), ("a", "<u4"), ("b", "<u4"), ("pad", "<u4"),
                        ("normal", "<f4", 4), ("depth", "<f4"), ("pad2", "<f4", 3),
                        ("point_a", "<f4", 4), ("point_b", "<f4", 4)])
BODY_STATE = np.dtype([("vel", "<f4", 4), ("ang", "<f4", 4), ("prev_vel", "<f4", 4),
                       ("inv_moment", "<f4", 4), ("inv_mass", "<f4"), ("friction", "<f4"),
                       ("pad", "<f4", 2)])
CONTACT = np.dtype([("a", "<u4"), ("b", "<u4"), ("friction", "<f4"), ("pad", "<f4"),
                    ("normal", "<f4", 4), ("tangent1", "<f4", 4), ("tangent2", "<f4", 4),
                    ("r_a", "<f4", 4), ("r_b", "<f4", 4), ("c0", "<f4", 4),
                    ("penalty", "<f4", 4), ("lambda", "<f4", 4)])
CONSTRAINT = np.dtype([("a", "<u4"), ("b", "<u4"), ("kind", "<u4"), ("pad", "<u4"),
                       ("anchor_a", "<f4", 4), ("anchor_b", "<f4", 4)])

assert SHAPE.itemsize == 80 and BODY.itemsize == 112 and PAIR.itemsize == 8
assert CONTACT_OUT.itemsize == 80 and BODY_STATE.itemsize == 80
assert CONTACT.itemsize == 144 and CONSTRAINT.itemsize == 48

_u32 = ctypes.c_uint32
_f32 = ctypes.c_float
_vp = ctypes.c_void_p


class RunOptions(ctypes.Structure):
    _fields_ = [("dt", _f32), ("gravity", _f32 * 3), ("alpha", _f32), ("beta_lin", _f32),
                ("penalty_max", _f32), ("iterations", _u32)]


class AvbdOptions(ctypes.Structure):
    _fields_ = [("dt", _f32), ("gravity", _f32 * 3), ("iterations", _u32), ("alpha", _f32),
                ("beta_lin", _f32), ("margin", _f32), ("penalty_min", _f32),
                ("penalty_max", _f32), ("gamma", _f32), ("friction", _f32)]


class Container(ctypes.Structure):
    _fields_ = [("center", _f32 * 3), ("half_extent", _f32), ("rotation", _f32 * 4)]


class AvbdResult(ctypes.Structure):
    _fields_ = [("positions", _vp), ("orientations", _vp), ("velocities", _vp),
                ("angular_velocities", _vp), ("prev_velocities", _vp), ("lambda_", _vp),
                ("penalty", _vp)]


class Capacity(ctypes.Structure):
    _fields_ = [("max_bodies", _u32), ("max_pairs", _u32), ("max_contacts", _u32),
                ("max_joints", _u32), ("max_scenes", _u32), ("max_hull_vertices", _u32)]


class Config(ctypes.Structure):
    _fields_ = [("solver_mode", _u32), ("precision", _u32), ("contacts_per_pair", _u32),
                ("use_graph", _u32), ("primal_variant", _u32), ("block_size", _u32),
                ("batched_solver", _u32), ("profile", _u32), ("broad_phase", _u32),
                ("bvh_rebuild_period", _u32), ("contact_lag", _u32), ("debug_flags", _u32)]


class WorldDesc(ctypes.Structure):
    _fields_ = [("n_bodies", _u32), ("n_constraints", _u32), ("n_scenes", _u32),
                ("n_hull_vertices", _u32), ("bodies", _vp), ("state", _vp), ("constraints", _vp),
                ("scene_offsets", _vp), ("containers", _vp), ("hull_vertices", _vp),
                ("positions_f64", _vp), ("orientations_f64", _vp)]


class StepStats(ctypes.Structure):
    _fields_ = [("pairs", _u32), ("contacts", _u32), ("colors", _u32), ("error_flags", _u32),
                ("steps", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64), ("primal_launches", _u32),
                ("dual_launches", _u32), ("primal_ms", ctypes.c_double), ("dual_ms", ctypes.c_double),
                ("broad_ms", ctypes.c_double), ("narrow_ms", ctypes.c_double), ("rows_ms", ctypes.c_double),
                ("solve_ms", ctypes.c_double), ("chunk_launches", _u32), ("pad", _u32), ("chunk_ms", ctypes.c_double)]


# every symbol include/*.h declares, with its argument types
_P = _vp
_PROTOS = {
    "dio_ctx_create": [ctypes.POINTER(Capacity), ctypes.POINTER(_vp)],
    "dio_ctx_destroy": [_P],
    "dio_status_string": [ctypes.c_int],
    "dio_ctx_last_error": [_P],
    "dio_ctx_configure": [_P, ctypes.POINTER(Config)],
    "dio_ctx_get_config": [_P, ctypes.POINTER(Config)],
    "dio_ctx_set_stream": [_P, _vp],
    "dio_ctx_synchronize": [_P],
    "dio_broad_submit": [_P, _vp, _u32],
    "dio_broad_pair_count": [_P, ctypes.POINTER(_u32)],
    "dio_read_pairs": [_P, _vp, _u32, ctypes.POINTER(_u32)],
    "dio_narrow_submit_pairs": [_P, _vp, _u32, _vp, _u32],
    "dio_narrow_submit": [_P, _u32],
    "dio_narrow_read": [_P, _vp, _u32, ctypes.POINTER(_u32)],
    "dio_set_hull_vertices": [_P, _vp, _u32],
    "dio_prepare_contacts": [_P, _vp, _vp, _u32, _vp, _u32, _vp, _u32, _vp,
                             ctypes.POINTER(AvbdOptions), _vp, _u32, ctypes.POINTER(_u32), _vp,
                             _vp, _u32],
    "dio_avbd_submit": [_P, _vp, _vp, _vp, _u32, _vp, _u32, _vp, _u32, _vp, _vp,
                        ctypes.POINTER(RunOptions)],
    "dio_avbd_read": [_P, ctypes.POINTER(AvbdResult)],
    "dio_avbd_solve_noalloc": [_vp, _vp, _vp, _u32, _vp, _u32, _vp, _u32, _vp, _vp, ctypes.POINTER(RunOptions),
                               _vp, _vp, _vp, _vp],
    "dio_world_upload": [_P, ctypes.POINTER(WorldDesc)],
    "dio_step": [_P, ctypes.POINTER(AvbdOptions), _u32],
    "dio_world_set_state": [_P, _vp, _vp],
    "dio_world_download": [_P, _vp, _vp],
    "dio_world_download_f64": [_P, _vp, _vp],
    "dio_world_contacts": [_P, _vp, _u32, ctypes.POINTER(_u32)],
    "dio_world_colors": [_P, _vp, _u32, ctypes.POINTER(_u32)],
    "dio_world_stats": [_P, ctypes.POINTER(StepStats)],
    "dio_world_reset_timers": [_P],
    "dio_world_export_transforms": [_P, _u32, _vp, _vp, ctypes.c_size_t],
    "dio_step_async": [_P, ctypes.POINTER(AvbdOptions), _u32],
    "dio_world_download_async": [_P, _vp, _vp],
    "dio_worlds_step_host": [ctypes.POINTER(_P), _u32, ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                             ctypes.POINTER(AvbdOptions), _u32],
    "dio_world_set_motion": [_P, _vp],
    "dio_world_download_motion": [_P, _vp],
    "dio_world_download_motion_async": [_P, _vp],
    "dio_worlds_step_motion_host": [ctypes.POINTER(_P), _u32, ctypes.POINTER(_vp), ctypes.POINTER(AvbdOptions),
                                    _u32],
    "dio_world_checkpoint": [_P, _vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)],
    "dio_world_resume": [_P, _vp, ctypes.c_size_t],
    "dio_autotune": [_P, ctypes.POINTER(AvbdOptions), _u32, ctypes.c_char_p, ctypes.POINTER(Config)],
    # include/dio_selftest.h: the device prefix sum and radix sort on host arrays
    "dio_selftest_scan": [_vp, _vp, _u32, _u32, _u32, ctypes.POINTER(_u32)],
    "dio_selftest_sort_u32": [_vp, _vp, _u32, _u32, _u32, _vp, _vp],
    "dio_selftest_sort_u64": [_vp, _vp, _u32, _u32, _u32, _vp, _vp],
}

_LIB = None


def lib():
    """Load libdio_cuda.so (built by diomedes_gb300.build); raise if absent."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m diomedes_gb300.build` "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _PROTOS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.dio_status_string.restype = ctypes.c_char_p
        L.dio_ctx_last_error.restype = ctypes.c_char_p
        _LIB = L
    return _LIB


def ptr(a):
    """Raw data pointer of a numpy array (None for None / empty)."""
    if a is None:
        return None
    return a.ctypes.data if a.size else None


class DioError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


def check(status, ctx=None, what=""):
    if status != DIO_OK:
        L = lib()
        detail = L.dio_status_string(status).decode()
        if ctx:
            last = L.dio_ctx_last_error(ctx)
            if last:
                detail += ": " + last.decode()
        raise DioError(status, f"{what}: {detail}" if what else detail)
    return status
