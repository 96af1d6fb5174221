"""The oracle: ctypes binding of oracle/tfx_oracle.cpp (CPU restatement of the reference shaders).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by __graft_entry__.smoke() as the checker, and by
bench.py's CPU-baseline / reference legs.  The shipped library never loads it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import OUT as LIB_PATH, build

_lib = None

STAGE_INTEGRATE = 1
STAGE_STRAND_LEVEL = 2
STAGE_VSP = 3
STAGE_LOCAL_SHAPE = 4
STAGE_LENGTH_WIND = 5
STAGE_FOLLOW = 6


class HairStruct(C.Structure):
    _fields_ = [("num_guide_strands", C.c_int32), ("verts_per_strand", C.c_int32), ("follow_per_guide", C.c_int32),
                ("_pad", C.c_int32), ("pos", C.c_void_p), ("prev", C.c_void_p), ("prevprev", C.c_void_p),
                ("tan", C.c_void_p), ("sld", C.c_void_p), ("init", C.c_void_p), ("rest", C.c_void_p),
                ("follow_offset", C.c_void_p), ("skin", C.c_void_p)]


class Settings(C.Structure):
    """TressFXSimulationSettings (TressFXSettings.h:59-87), field for field."""
    _fields_ = [("vsp_coeff", C.c_float), ("vsp_accel_threshold", C.c_float),
                ("local_constraint_stiffness", C.c_float), ("local_constraints_iterations", C.c_int32),
                ("global_constraint_stiffness", C.c_float), ("global_constraints_range", C.c_float),
                ("length_constraints_iterations", C.c_int32), ("damping", C.c_float),
                ("gravity_magnitude", C.c_float), ("tip_separation", C.c_float), ("wind_magnitude", C.c_float),
                ("wind_direction", C.c_float * 3), ("wind_angle_radians", C.c_float),
                ("clamp_position_delta", C.c_float)]


class SimParams(C.Structure):
    """TressFXSimulationParams (TressFXConstantBuffers.h:41-85): the 160-byte header, then 512 bone
    matrices (16 floats each, row-major)."""
    _fields_ = [("header", C.c_uint8 * 160), ("bones", C.c_float * (512 * 16))]

    def header_bytes(self) -> bytes:
        return bytes(self.header)

    def bones_view(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.bones).reshape(512, 16)

    def set_reset(self, value: float) -> None:
        C.c_float.from_buffer(self.header, 144).value = value


class SdfParams(C.Structure):
    _fields_ = [("origin", C.c_float * 4), ("cell_size", C.c_float), ("nx", C.c_int32), ("ny", C.c_int32),
                ("nz", C.c_int32)]


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(str(LIB_PATH))
        vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
        for suf in ("f32", "f64"):
            getattr(l, f"tfxo_stage_{suf}").argtypes = [i32, C.POINTER(HairStruct), vp, i32]
            getattr(l, f"tfxo_simulate_{suf}").argtypes = [C.POINTER(HairStruct), vp, i32, i32]
            getattr(l, f"tfxo_sdf_build_{suf}").argtypes = [vp, vp, vp, vp, i64, i32]
            getattr(l, f"tfxo_sdf_collide_{suf}").argtypes = [vp, vp, C.c_float, C.POINTER(HairStruct), i32]
        l.tfxo_sdf_construct_f32.argtypes = [vp, vp, vp, vp, i64, i32]
        l.tfxo_settings_default.argtypes = [C.POINTER(Settings)]
        l.tfxo_fill_sim_params.argtypes = [C.POINTER(Settings), C.c_float, i32, i32, i32, C.POINTER(SimParams)]
        l.tfxo_fill_sim_params.restype = C.c_int
        l.tfxo_signed_distance_triangle_f32.argtypes = [vp, vp, vp, vp]
        l.tfxo_signed_distance_triangle_f32.restype = C.c_float
        l.tfxo_float_flip3.argtypes = [C.c_float]
        l.tfxo_float_flip3.restype = C.c_uint32
        l.tfxo_ifloat_flip3.argtypes = [C.c_uint32]
        l.tfxo_ifloat_flip3.restype = C.c_uint32
        l.tfxo_mesh_skin_f32.argtypes = [vp, vp, vp, vp, i64, i32]
        l.tfxo_sdf_collide_mixed_f32.argtypes = [vp, vp, C.c_float, C.POINTER(HairStruct), i32]
        l.tfxo_marching_cubes_f32.argtypes = [vp, vp, C.c_float, vp, vp, i32, vp, vp]
        _lib = l
    return _lib


def _p(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


class OracleHair:
    """Host copy of one hair object's buffers in float32 or float64, updated by the oracle."""

    def __init__(self, asset, dtype=np.float32):
        self.dtype = np.dtype(dtype)
        self.G, self.n, self.F = asset.num_guide_strands, asset.verts_per_strand, asset.follow_per_guide
        S = self.G * (self.F + 1)
        cv = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float32).astype(self.dtype))  # noqa: E731
        self.pos = cv(asset.positions).copy()
        self.prev = cv(asset.positions).copy()
        self.prevprev = cv(asset.positions).copy()
        self.tan = cv(asset.tangents).copy()
        self.sld = np.zeros((S, 12), dtype=self.dtype)
        self.init = cv(asset.positions).copy()
        self.rest = cv(asset.rest_lengths).copy()
        self.follow_offset = cv(asset.follow_root_offsets).copy()
        self.skin = cv(asset.bone_skinning).copy()
        self._struct = self._make_struct()

    def _make_struct(self) -> HairStruct:
        return HairStruct(self.G, self.n, self.F, 0, _p(self.pos), _p(self.prev), _p(self.prevprev), _p(self.tan),
                          _p(self.sld), _p(self.init), _p(self.rest), _p(self.follow_offset), _p(self.skin))

    @property
    def suffix(self) -> str:
        return "f32" if self.dtype == np.float32 else "f64"

    def stage(self, stage: int, params, threads: int = 0) -> None:
        r = getattr(lib(), f"tfxo_stage_{self.suffix}")(stage, C.byref(self._struct), C.addressof(params), threads)
        if r:
            raise RuntimeError(f"oracle stage {stage} failed: {r}")

    def simulate(self, params, cpu_local_iterations: int, threads: int = 0) -> None:
        r = getattr(lib(), f"tfxo_simulate_{self.suffix}")(C.byref(self._struct), C.addressof(params),
                                                           cpu_local_iterations, threads)
        if r:
            raise RuntimeError(f"oracle simulate failed: {r}")

    def state(self) -> dict[str, np.ndarray]:
        return {"pos": self.pos.copy(), "prev": self.prev.copy(), "prevprev": self.prevprev.copy(),
                "tan": self.tan.copy(), "sld": self.sld.copy()}

    def load_state(self, st: dict[str, np.ndarray]) -> None:
        for k, v in st.items():
            getattr(self, k)[...] = np.asarray(v).astype(self.dtype).reshape(getattr(self, k).shape)


def sdf_params(grid) -> SdfParams:
    p = SdfParams()
    for i in range(4):
        p.origin[i] = grid.origin[i]
    p.cell_size = grid.cell_size
    p.nx, p.ny, p.nz = grid.num_cells_x, grid.num_cells_y, grid.num_cells_z
    return p


def sdf_build(grid, mesh_vertices: np.ndarray, indices: np.ndarray, dtype=np.float32, threads: int = 0) -> np.ndarray:
    """Initialize + Construct + Finalize; returns the grid as uint32 (f32) or uint64 (f64) words."""
    gp = sdf_params(grid)
    cells = gp.nx * gp.ny * gp.nz
    out = np.zeros(cells, dtype=np.uint32 if np.dtype(dtype) == np.float32 else np.uint64)
    mv = np.ascontiguousarray(mesh_vertices, dtype=np.float32)
    ix = np.ascontiguousarray(indices, dtype=np.uint32)
    suf = "f32" if np.dtype(dtype) == np.float32 else "f64"
    r = getattr(lib(), f"tfxo_sdf_build_{suf}")(_p(out), C.addressof(gp), _p(mv), _p(ix), len(ix) // 3, threads)
    if r:
        raise RuntimeError(f"oracle sdf build failed: {r}")
    return out


def sdf_construct(grid, words: np.ndarray, mesh_vertices: np.ndarray, indices: np.ndarray, threads: int = 0) -> None:
    gp = sdf_params(grid)
    mv = np.ascontiguousarray(mesh_vertices, dtype=np.float32)
    ix = np.ascontiguousarray(indices, dtype=np.uint32)
    lib().tfxo_sdf_construct_f32(_p(words), C.addressof(gp), _p(mv), _p(ix), len(ix) // 3, threads)


def sdf_collide(grid, sdf_words: np.ndarray, margin: float, hair: OracleHair, threads: int = 0) -> None:
    gp = sdf_params(grid)
    r = getattr(lib(), f"tfxo_sdf_collide_{hair.suffix}")(_p(sdf_words), C.addressof(gp), float(margin),
                                                          C.byref(hair._struct), threads)
    if r:
        raise RuntimeError(f"oracle collide failed: {r}")


def sdf_collide_mixed(grid, sdf_words: np.ndarray, margin: float, hair: OracleHair, threads: int = 0) -> None:
    """CollideHairVerticesWithSdf (mixed forward / backward differences) on every vertex."""
    gp = sdf_params(grid)
    r = lib().tfxo_sdf_collide_mixed_f32(_p(sdf_words), C.addressof(gp), float(margin), C.byref(hair._struct), threads)
    if r:
        raise RuntimeError(f"oracle mixed collide failed: {r}")


def marching_cubes(grid, sdf: np.ndarray, iso: float, edge_table: np.ndarray, tri_table: np.ndarray,
                   max_vertices: int) -> tuple[np.ndarray, int]:
    """RunMarchingCubesOnSdf in cell-index order: ({position, normal}[max_vertices] as (max, 8) float32,
    the counter).  `iso` is the world-unit iso value (cell size * iso level)."""
    gp = sdf_params(grid)
    f = np.ascontiguousarray(np.asarray(sdf).view(np.float32) if np.asarray(sdf).dtype == np.uint32 else sdf,
                             dtype=np.float32)
    e = np.ascontiguousarray(edge_table, dtype=np.int32)
    t = np.ascontiguousarray(tri_table, dtype=np.int32).reshape(-1)
    out = np.zeros((max_vertices, 8), np.float32)
    cnt = np.zeros(1, np.int32)
    r = lib().tfxo_marching_cubes_f32(_p(f), C.addressof(gp), float(np.float32(iso)), _p(e), _p(t), int(max_vertices),
                                      _p(out), _p(cnt))
    if r:
        raise RuntimeError(f"oracle marching cubes failed: {r}")
    return out, int(cnt[0])


def mesh_skin(vertices: np.ndarray, skinning: np.ndarray, bones: np.ndarray, threads: int = 0) -> np.ndarray:
    v = np.ascontiguousarray(vertices, dtype=np.float32)
    s = np.ascontiguousarray(skinning, dtype=np.float32)
    full = np.zeros((512, 16), dtype=np.float32)
    b = np.asarray(bones, dtype=np.float32).reshape(-1, 16)
    full[:len(b)] = b
    out = np.zeros_like(v)
    r = lib().tfxo_mesh_skin_f32(_p(out), _p(v), _p(s), _p(full), len(v), threads)
    if r:
        raise RuntimeError("oracle mesh skin failed")
    return out


def signed_distance_triangle(p, x0, x1, x2) -> float:
    a = [np.ascontiguousarray(np.asarray(v, dtype=np.float32)) for v in (p, x0, x1, x2)]
    return float(lib().tfxo_signed_distance_triangle_f32(*[_p(v) for v in a]))


def float_flip3(f: float) -> int:
    return int(lib().tfxo_float_flip3(f))


def ifloat_flip3(u: int) -> int:
    return int(lib().tfxo_ifloat_flip3(u))


def settings(**overrides) -> Settings:
    """The reference's default settings, then the given fields (names as in the Settings struct)."""
    st = Settings()
    lib().tfxo_settings_default(C.byref(st))
    for k, v in overrides.items():
        if k == "wind_direction":
            for i in range(3):
                st.wind_direction[i] = float(v[i])
        else:
            setattr(st, k, v)
    return st


def fill_sim_params(params: SimParams, st: Settings, dt: float, n: int, F: int, frame: int) -> int:
    """UpdateSimulationParameters on `params`; returns the CPU local-shape iteration count."""
    return int(lib().tfxo_fill_sim_params(C.byref(st), float(dt), int(n), int(F), int(frame), C.byref(params)))
