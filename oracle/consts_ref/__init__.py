"""The reference's own per-frame constant code, compiled here (test infrastructure, a checker only).

TressFXHairObject::UpdateSimulationParameters and SetWind (src/TressFX/TressFXHairObject.cpp:172-235,
380-437) fill the simulation constant block.  TressFXHairObject.cpp as a whole needs the engine
interface and does not build here, so build.py copies the text of those functions out of the
reference tree (at build time, into the git-ignored oracle/_ref/) and compiles it, unchanged, inside a
minimal stand-in for the class, linked with the reference's src/Math/Vector3D.cpp, Quaternion.cpp and
Matrix33.cpp.  tests/test_consts_pin.py compares the library's tfx_fill_sim_params and the oracle's
restatement with it bit for bit; tests/golden/make_consts_golden.py writes its outputs to a fixture
for machines without the reference tree.
"""
from __future__ import annotations

import ctypes as C

from .build import LIB, available, build  # noqa: F401

_lib = None

HEADER_BYTES = 160   # TressFXSimulationParams before the bone matrices


class RefSettings(C.Structure):
    """TressFXSimulationSettings' fields in declaration order (TressFXSettings.h:59-87)."""
    _fields_ = [("vsp_coeff", C.c_float), ("vsp_accel_threshold", C.c_float),
                ("local_constraint_stiffness", C.c_float), ("local_constraints_iterations", C.c_int32),
                ("global_constraint_stiffness", C.c_float), ("global_constraints_range", C.c_float),
                ("length_constraints_iterations", C.c_int32), ("damping", C.c_float),
                ("gravity_magnitude", C.c_float), ("tip_separation", C.c_float), ("wind_magnitude", C.c_float),
                ("wind_direction", C.c_float * 3), ("wind_angle_radians", C.c_float),
                ("clamp_position_delta", C.c_float)]


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build()
        if path is None:
            raise FileNotFoundError("the reference tree is not present and no built copy exists")
        l = C.CDLL(str(path))
        l.ref_settings_default.argtypes = [C.POINTER(RefSettings)]
        l.ref_update_simulation_parameters.argtypes = [C.POINTER(RefSettings), C.c_float, C.c_int, C.c_int, C.c_int,
                                                       C.c_void_p, C.POINTER(C.c_int32)]
        l.ref_update_simulation_parameters.restype = C.c_int
        _lib = l
    return _lib


def settings(**overrides) -> RefSettings:
    """The reference's default settings (its constructor), then the given fields."""
    s = RefSettings()
    lib().ref_settings_default(C.byref(s))
    for k, v in overrides.items():
        if k == "wind_direction":
            for i in range(3):
                s.wind_direction[i] = float(v[i])
        else:
            setattr(s, k, v)
    return s


def update_simulation_parameters(s: RefSettings, dt: float, n: int, F: int, frame: int) -> tuple[bytes, int]:
    """(the 160-byte header of m_SimCB[frame % 2] after UpdateSimulationParameters, CPU local iterations)
    for an object created at frame 0 and advanced to `frame` (its constant blocks start zeroed)."""
    buf = C.create_string_buffer(HEADER_BYTES)
    it = C.c_int32()
    r = lib().ref_update_simulation_parameters(C.byref(s), float(dt), int(n), int(F), int(frame), buf, C.byref(it))
    if r:
        raise RuntimeError(f"ref_update_simulation_parameters failed: {r}")
    return buf.raw, it.value


class ReferenceConstants:
    """The host half of TressFXHairObject with the reference's own UpdateSimulationParameters: two
    constant blocks by frame parity, the frame counter, the reset flag (TressFXHairObject.h:104, 129)
    and the CPU local-shape iteration count.  The same interface as oracle.scene_driver's
    OracleConstants."""

    def __init__(self, n: int, F: int):
        from oracle import SimParams
        self.n, self.F = n, F
        self.blocks = [SimParams(), SimParams()]
        self.frame = 0
        self.cpu_local_iterations = 0
        self.blocks[0].set_reset(1.0)

    def update_simulation_parameters(self, overrides: dict, dt: float) -> None:
        # every header word UpdateSimulationParameters writes, plus the reset flag as the object holds it
        hdr, self.cpu_local_iterations = update_simulation_parameters(settings(**overrides), dt, self.n, self.F,
                                                                      self.frame)
        C.memmove(self.blocks[self.frame % 2].header, hdr, HEADER_BYTES)

    def update_bone_matrices(self, mats) -> None:
        import numpy as np
        mats = np.ascontiguousarray(mats, dtype=np.float32).reshape(-1, 16)
        k = min(len(mats), 512)
        self.blocks[self.frame % 2].bones_view()[:k] = mats[:k]

    def increase_simulation_frame(self) -> None:
        self.blocks[self.frame % 2].set_reset(0.0)
        self.frame += 1

    def current_params(self):
        return self.blocks[self.frame % 2]
