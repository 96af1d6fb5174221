"""The reference's own compute shaders, compiled as C++ (test infrastructure).

``build()`` runs translate.py over the HLSL files of the reference checkout and compiles them with
hlsl_shim.h and driver.cpp into oracle/_ref/libtfx_hlsl_ref.so.  It needs the reference sources,
so it runs where they are mounted (never on a machine without them); the golden fixtures under
tests/golden/ carry its outputs everywhere else.

``RefPipeline`` drives those kernels in the sample's per-frame order with the reference's own
dispatch sizes, over host copies of the buffers.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE.parent / "_ref"
LIB = REF_DIR / "libtfx_hlsl_ref.so"
SHADER_ROOT = Path(os.environ.get("TFX_REFERENCE", "/root/reference"))

_lib = None


def available() -> bool:
    return (SHADER_ROOT / "src" / "Shaders" / "TressFXSimulation.hlsl").exists()


def build(force: bool = False) -> Path:
    from . import translate
    deps = [HERE / "hlsl_shim.h", HERE / "driver.cpp", HERE / "translate.py"]
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return LIB
    translate.main(REF_DIR)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math",
           "-fno-strict-aliasing", "-fPIC", "-shared", "-w", f"-I{HERE}", f"-I{REF_DIR}",
           f"-I{SHADER_ROOT / 'src'}", "-o", str(tmp),
           str(HERE / "driver.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference shader build failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(str(LIB))
        vp = C.c_void_p
        l.tfxr_sim_dispatch.argtypes = [C.c_int, vp, vp]
        l.tfxr_sdf_update.argtypes = [vp, C.c_int64, vp, vp, C.c_int, vp, C.c_int]
        l.tfxr_sdf_collide.argtypes = [vp, C.c_int64, vp, C.c_float, vp]
        l.tfxr_sdf_collide_mixed.argtypes = [vp, C.c_int64, vp, C.c_float, vp]
        l.tfxr_expand_strands.argtypes = [vp, vp, C.c_int64, vp, vp, vp, vp, vp, C.c_int, vp]
        l.tfxr_mesh_skin.argtypes = [vp, vp, vp, vp, C.c_int]
        l.tfxr_mc_tables.argtypes = [vp, vp]
        l.tfxr_marching_cubes.argtypes = [vp, C.c_int64, vp, C.c_float, vp, vp, C.c_int, vp, vp]
        _lib = l
    return _lib


class RefPipeline:
    """Sample frame order over the reference kernels (float32 host buffers)."""

    def __init__(self, scene):
        import oracle
        from oracle.consts_ref import ReferenceConstants
        from oracle.scene_driver import margin_world
        self._margin_world = margin_world
        self.scene = scene
        self.hair = [oracle.OracleHair(o.asset) for o in scene.objects]
        self.consts = [ReferenceConstants(o.asset.verts_per_strand, o.asset.follow_per_guide) for o in scene.objects]
        self.sdf_words = [None] * len(scene.objects)
        self.skinned = [None] * len(scene.objects)
        self.frame = 0

    def stage(self, i: int, kernel: int) -> None:
        c = self.consts[i]
        r = lib().tfxr_sim_dispatch(kernel, C.addressof(self.hair[i]._struct), C.addressof(c.current_params()))
        if r:
            raise RuntimeError("reference dispatch failed")

    def skin_and_build(self, i: int, fin) -> None:
        import oracle
        o = self.scene.objects[i]
        v = np.ascontiguousarray(o.mesh.vertices, dtype=np.float32)
        out = v.copy()
        bones = np.zeros((512, 16), dtype=np.float32)
        b = np.asarray(fin.mesh_bones[i], dtype=np.float32).reshape(-1, 16)
        bones[:len(b)] = b
        sk = np.ascontiguousarray(o.mesh.skinning, dtype=np.float32)
        lib().tfxr_mesh_skin(out.ctypes.data, v.ctypes.data, sk.ctypes.data, bones.ctypes.data, len(v))
        self.skinned[i] = out
        g = fin.grids[i]
        alloc = int(np.float32(1.4) * np.float32(g.num_cells))
        alloc = max(alloc, g.num_cells)
        words = np.zeros(alloc, dtype=np.uint32)
        gp = oracle.sdf_params(g)
        idx = np.ascontiguousarray(o.mesh.indices, dtype=np.uint32)
        lib().tfxr_sdf_update(words.ctypes.data, alloc, C.addressof(gp), out.ctypes.data, len(out), idx.ctypes.data,
                              len(idx) // 3)
        self.sdf_words[i] = words[:g.num_cells].copy()
        self._alloc_words = words

    def collide(self, i: int, fin) -> None:
        import oracle
        o = self.scene.objects[i]
        g = fin.grids[i]
        words = np.zeros(max(int(np.float32(1.4) * np.float32(g.num_cells)), g.num_cells), dtype=np.uint32)
        words[:g.num_cells] = self.sdf_words[i]
        gp = oracle.sdf_params(g)
        lib().tfxr_sdf_collide(words.ctypes.data, len(words), C.addressof(gp), self._margin_world(o, g),
                               C.addressof(self.hair[i]._struct))

    def step(self, fin, per_stage=None) -> None:
        sc = self.scene
        for i, c in enumerate(self.consts):
            c.update_simulation_parameters(fin.settings_overrides[i], sc.dt)
            c.update_bone_matrices(fin.hair_bones[i])
        for i, o in enumerate(sc.objects):
            if o.mesh is not None:
                self.skin_and_build(i, fin)
        for k in (1, 2, 3, 4, 5, 6):
            for i, c in enumerate(self.consts):
                reps = c.cpu_local_iterations if k == 4 else 1
                for _ in range(reps):
                    self.stage(i, k)
            if per_stage is not None:
                per_stage(k, self)
        for c in self.consts:
            c.increase_simulation_frame()
        for i, o in enumerate(sc.objects):
            if o.mesh is not None:
                self.collide(i, fin)
        self.frame += 1
