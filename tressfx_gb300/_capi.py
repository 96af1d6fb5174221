"""ctypes binding of the C ABI in include/tressfx_gb300.h (libtfxgb300.so).

The library is the product; this module only declares its structs and entry points for Python
callers (tests, benchmarks, tools).  Loading fails loudly when the library has not been built:
there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libtfxgb300.so"

TFX_MAX_BONES = 512
TFX_THREAD_GROUP_SIZE = 64

# status codes
TFX_OK = 0
TFX_ERR_INVALID_ARGUMENT = 1
TFX_ERR_VERTS_PER_STRAND = 2
TFX_ERR_BONE_INDEX = 3
TFX_ERR_BONE_WEIGHTS = 4
TFX_ERR_CUDA = 5
TFX_ERR_OUT_OF_MEMORY = 6
TFX_ERR_TIMEOUT = 7
TFX_ERR_SIZE = 8
TFX_ERR_MISMATCH = 9
TFX_ERR_NO_DEVICE = 10

# kernel ids
K_INTEGRATION_AND_GLOBAL_SHAPE = 1
K_STRAND_LEVEL_DATA = 2
K_VELOCITY_SHOCK_PROPAGATION = 3
K_LOCAL_SHAPE_CONSTRAINTS = 4
K_LENGTH_WIND_COLLISION = 5
K_UPDATE_FOLLOW_HAIR = 6
K_SDF_INITIALIZE = 7
K_SDF_CONSTRUCT = 8
K_SDF_FINALIZE = 9
K_SDF_COLLIDE = 10
K_MESH_BONE_SKINNING = 11

# buffer ids
BUF_POSITIONS = 1
BUF_POSITIONS_PREV = 2
BUF_POSITIONS_PREV_PREV = 3
BUF_TANGENTS = 4
BUF_STRAND_LEVEL_DATA = 5
BUF_INITIAL_POSITIONS = 6
BUF_REST_LENGTHS = 7
BUF_FOLLOW_ROOT_OFFSETS = 8
BUF_BONE_SKINNING = 9


class SimParams(C.Structure):
    """TressFXSimulationParams (src/TressFX/TressFXConstantBuffers.h:41-85)."""
    _fields_ = [
        ("wind", C.c_float * 4), ("wind1", C.c_float * 4), ("wind2", C.c_float * 4), ("wind3", C.c_float * 4),
        ("shape", C.c_float * 4), ("grav_time_tip", C.c_float * 4),
        ("sim_ints", C.c_int32 * 4), ("counts", C.c_int32 * 4), ("vsp", C.c_float * 4),
        ("reset_positions", C.c_float), ("clamp_position_delta", C.c_float), ("pad1", C.c_float), ("pad2", C.c_float),
        ("bone_matrices", (C.c_float * 16) * TFX_MAX_BONES),
    ]

    def bones_view(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.bone_matrices).reshape(TFX_MAX_BONES, 16)

    def copy(self) -> "SimParams":
        c = SimParams()
        C.memmove(C.addressof(c), C.addressof(self), C.sizeof(SimParams))
        return c


assert C.sizeof(SimParams) == 160 + 512 * 64


class SimSettings(C.Structure):
    """TressFXSimulationSettings (src/TressFX/TressFXSettings.h:35-87)."""
    _fields_ = [
        ("vsp_coeff", C.c_float), ("vsp_accel_threshold", C.c_float),
        ("local_constraint_stiffness", C.c_float), ("local_constraints_iterations", C.c_int32),
        ("global_constraint_stiffness", C.c_float), ("global_constraints_range", C.c_float),
        ("length_constraints_iterations", C.c_int32), ("damping", C.c_float), ("gravity_magnitude", C.c_float),
        ("tip_separation", C.c_float), ("wind_magnitude", C.c_float), ("wind_direction", C.c_float * 3),
        ("wind_angle_radians", C.c_float), ("clamp_position_delta", C.c_float),
    ]


class HairDesc(C.Structure):
    _fields_ = [("num_guide_strands", C.c_int32), ("verts_per_strand", C.c_int32),
                ("follow_hairs_per_guide", C.c_int32), ("reserved", C.c_int32)]


class StrandParams(C.Structure):
    """TressFXStrandParams (cbuffer TressFXStrandParameters, TressFXRendering.hlsl:61-80)."""
    _fields_ = [("mat_base_color", C.c_float * 4), ("mat_tip_color", C.c_float * 4), ("tip_percentage", C.c_float),
                ("strand_uv_tiling_factor", C.c_float), ("fiber_ratio", C.c_float), ("fiber_radius", C.c_float),
                ("num_vertices_per_strand", C.c_int32), ("enable_thin_tip", C.c_int32), ("node_pool_size", C.c_int32),
                ("render_params_index", C.c_int32), ("enable_strand_uv", C.c_int32),
                ("enable_strand_tangent", C.c_int32), ("padding", C.c_int32 * 2)]


class SdfGrid(C.Structure):
    """Grid part of TressFXSDFCollisionParams (TressFXConstantBuffers.h:119-134)."""
    _fields_ = [("origin", C.c_float * 4), ("cell_size", C.c_float),
                ("num_cells_x", C.c_int32), ("num_cells_y", C.c_int32), ("num_cells_z", C.c_int32)]

    @property
    def dims(self) -> tuple[int, int, int]:
        return (self.num_cells_x, self.num_cells_y, self.num_cells_z)

    @property
    def num_cells(self) -> int:
        return self.num_cells_x * self.num_cells_y * self.num_cells_z


class NsdfDesc(C.Structure):
    _fields_ = [("box_min", C.c_float * 3), ("box_max", C.c_float * 3), ("cell_size", C.c_float),
                ("band_cells", C.c_float), ("pose_scale", C.c_float), ("sphere_center", C.c_float * 3),
                ("sphere_radius", C.c_float), ("seed", C.c_uint32), ("max_samples", C.c_int64),
                ("max_eval_samples", C.c_int64), ("contact_slack_cells", C.c_float)]


class TfxError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{status_name(status)}: {message}")
        self.status = status


_lib = None

P = C.c_void_p
I32 = C.c_int32
F32 = C.c_float
FP = C.POINTER(C.c_float)
U32P = C.POINTER(C.c_uint32)

_PROTOS = {
    "tfx_status_string": (C.c_char_p, [C.c_int]),
    "tfx_last_error": (C.c_char_p, []),
    "tfx_abi_version": (C.c_int, []),
    "tfx_sim_settings_default": (C.c_int, [C.POINTER(SimSettings)]),
    "tfx_fill_sim_params": (C.c_int, [C.POINTER(SimParams), C.POINTER(SimSettings), F32, C.c_int, C.c_int, C.c_int,
                                      C.POINTER(C.c_int32)]),
    "tfx_context_create": (C.c_int, [C.c_int, C.POINTER(P)]),
    "tfx_context_destroy": (C.c_int, [P]),
    "tfx_context_synchronize": (C.c_int, [P]),
    "tfx_context_stream": (P, [P]),
    "tfx_context_timestamp": (C.c_int, [P, C.c_char_p]),
    "tfx_context_timestamps": (C.c_int, [P, P, FP, C.c_int, C.POINTER(C.c_int)]),
    "tfx_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(P)]),
    "tfx_host_free": (C.c_int, [P]),
    "tfx_hair_create": (C.c_int, [P, C.POINTER(HairDesc), P, P, P, P, P, C.POINTER(P)]),
    "tfx_hair_destroy": (C.c_int, [P]),
    "tfx_hair_validate": (C.c_int, [C.POINTER(HairDesc), P]),
    "tfx_hair_update_constants": (C.c_int, [P, C.POINTER(SimParams), C.c_int]),
    "tfx_hair_dispatch": (C.c_int, [P, C.c_int, C.c_int]),
    "tfx_hair_simulate": (C.c_int, [P, C.c_int]),
    "tfx_hair_read": (C.c_int, [P, C.c_int, P, C.c_size_t]),
    "tfx_hair_write": (C.c_int, [P, C.c_int, P, C.c_size_t]),
    "tfx_hair_read_async": (C.c_int, [P, C.c_int, P, C.c_size_t]),
    "tfx_hair_write_async": (C.c_int, [P, C.c_int, P, C.c_size_t]),
    "tfx_hair_get_buffer": (C.c_int, [P, C.c_int, C.POINTER(P), C.POINTER(C.c_size_t)]),
    "tfx_hair_get_counts": (C.c_int, [P, C.POINTER(C.c_int32)]),
    "tfx_hair_expand_strands": (C.c_int, [P, C.POINTER(StrandParams), FP, FP, FP, C.c_int, P]),
    "tfx_sdf_grid_from_bbox": (C.c_int, [FP, FP, C.c_int, C.POINTER(SdfGrid), FP, C.POINTER(C.c_int64)]),
    "tfx_sdf_grid_origin": (C.c_int, [FP, F32, C.POINTER(SdfGrid)]),
    "tfx_sdf_create": (C.c_int, [P, C.c_int64, C.POINTER(P)]),
    "tfx_sdf_destroy": (C.c_int, [P]),
    "tfx_sdf_set_mesh": (C.c_int, [P, P, C.c_int, P, C.c_int]),
    "tfx_sdf_update": (C.c_int, [P, C.POINTER(SdfGrid)]),
    "tfx_sdf_dispatch": (C.c_int, [P, C.c_int, C.POINTER(SdfGrid)]),
    "tfx_sdf_collide": (C.c_int, [P, P, C.POINTER(SdfGrid), F32]),
    "tfx_sdf_collide_mixed": (C.c_int, [P, P, C.POINTER(SdfGrid), F32]),
    "tfx_sdf_read": (C.c_int, [P, P, C.c_size_t]),
    "tfx_sdf_write": (C.c_int, [P, P, C.c_size_t]),
    "tfx_sdf_get_buffer": (C.c_int, [P, C.POINTER(P), C.POINTER(C.c_size_t)]),
    "tfx_sdf_build_static": (C.c_int, [P, P, P, C.c_int, P, C.c_int, P]),
    "tfx_mc_create": (C.c_int, [P, C.c_int, C.c_int64, C.POINTER(P)]),
    "tfx_mc_destroy": (C.c_int, [P]),
    "tfx_mc_default_tables": (C.c_int, [P, P]),
    "tfx_mc_set_tables": (C.c_int, [P, P, P]),
    "tfx_mc_set_iso_level": (C.c_int, [P, F32]),
    "tfx_mc_update": (C.c_int, [P, P, C.POINTER(SdfGrid)]),
    "tfx_mc_run": (C.c_int, [P, P, C.POINTER(SdfGrid)]),
    "tfx_mc_get_buffers": (C.c_int, [P, C.POINTER(P), C.POINTER(P)]),
    "tfx_mc_read": (C.c_int, [P, P, C.c_size_t, C.POINTER(C.c_int32)]),
    "tfx_mesh_create": (C.c_int, [P, P, C.c_int, P, C.c_int, P, C.POINTER(P)]),
    "tfx_mesh_destroy": (C.c_int, [P]),
    "tfx_mesh_skin": (C.c_int, [P, P, C.c_int]),
    "tfx_mesh_get_buffers": (C.c_int, [P, C.POINTER(P), C.POINTER(P), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "tfx_mesh_read_skinned": (C.c_int, [P, P, C.c_size_t]),
    "tfx_nsdf_create": (C.c_int, [P, C.POINTER(NsdfDesc), C.POINTER(P)]),
    "tfx_nsdf_destroy": (C.c_int, [P]),
    "tfx_nsdf_add_samples": (C.c_int, [P, C.c_int, P, P, C.POINTER(SdfGrid), P, C.c_int, FP, FP, C.c_int, F32]),
    "tfx_nsdf_train": (C.c_int, [P, C.c_int, C.c_int, F32, FP]),
    "tfx_nsdf_evaluate": (C.c_int, [P, C.c_int, P, P, P, C.c_int64, C.POINTER(C.c_int64)]),
    "tfx_nsdf_query": (C.c_int, [P, P, C.c_int, FP, P]),
    "tfx_nsdf_collide": (C.c_int, [P, P, P, C.POINTER(SdfGrid), F32, FP, C.POINTER(C.c_int32)]),
    "tfx_nsdf_get_params": (C.c_int, [P, P, C.c_size_t]),
    "tfx_nsdf_set_params": (C.c_int, [P, P, C.c_size_t]),
    "tfx_nsdf_set_inference": (C.c_int, [P, C.c_int]),
    "tfx_nsdf_set_samples": (C.c_int, [P, C.c_int, P, C.c_int64]),
    "tfx_nsdf_get_gradients": (C.c_int, [P, P, C.c_size_t]),
    "tfx_nsdf_get_info": (C.c_int, [P, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int32)]),
    "tfx_batch_create": (C.c_int, [P, C.POINTER(P)]),
    "tfx_batch_readback": (C.c_int, [P, C.POINTER(P), C.c_int, C.c_int, C.POINTER(C.c_int64)]),
    "tfx_batch_wait_readback": (C.c_int, [P, C.c_int64]),
    "tfx_batch_destroy": (C.c_int, [P]),
    "tfx_batch_add_sdf": (C.c_int, [P, P, P, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "tfx_batch_add_hair": (C.c_int, [P, P, C.c_int, C.POINTER(C.c_int)]),
    "tfx_batch_add_hair_collision": (C.c_int, [P, C.c_int, C.c_int]),
    "tfx_batch_build": (C.c_int, [P, C.c_int]),
    "tfx_batch_set_option": (C.c_int, [P, C.c_int, C.c_int]),
    "tfx_batch_get_option": (C.c_int, [P, C.c_int, C.POINTER(C.c_int)]),
    "tfx_batch_autotune": (C.c_int, [P, C.c_int]),
    "tfx_batch_set_hair_constants": (C.c_int, [P, C.c_int, C.POINTER(SimParams), C.c_int, C.c_int]),
    "tfx_batch_set_sdf_frame": (C.c_int, [P, C.c_int, C.POINTER(SdfGrid), F32]),
    "tfx_batch_set_mesh_bones": (C.c_int, [P, C.c_int, P, C.c_int]),
    "tfx_batch_run": (C.c_int, [P]),
    "tfx_batch_synchronize": (C.c_int, [P]),
    "tfx_hair_count_nonfinite": (C.c_int, [P, C.POINTER(C.c_int64)]),
    "tfx_batch_describe": (C.c_int, [P, C.c_char_p, C.c_size_t, C.POINTER(C.c_int32)]),
    "tfx_batch_profile_frame": (C.c_int, [P, FP, C.c_int, C.POINTER(C.c_int)]),
}

EXPORTED_SYMBOLS = tuple(_PROTOS)


def lib() -> C.CDLL:
    """Load libtfxgb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                              " (there is no CPU fallback)")
        l = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _PROTOS.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def status_name(s: int) -> str:
    try:
        return lib().tfx_status_string(s).decode()
    except Exception:  # pragma: no cover - only when the library itself is missing
        return f"status {s}"


def check(status: int, what: str = "") -> None:
    if status != TFX_OK:
        msg = lib().tfx_last_error().decode()
        raise TfxError(status, f"{what}: {msg}" if what else msg)


def ptr(a: np.ndarray | None) -> int | None:
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the C ABI must be C-contiguous"
    return a.ctypes.data
