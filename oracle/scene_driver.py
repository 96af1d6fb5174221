"""Oracle frame driver (test infrastructure): the sample's per-frame order on the CPU.

Mirrors tressfx_gb300.headless.PlainPipeline step for step -- skin meshes, rebuild SDFs,
simulate (stage-major over objects), collide -- with every kernel replaced by the oracle's
restatement.  The constant blocks are the oracle's own (tfxo_fill_sim_params, pinned bit for bit to
the reference's TressFXHairObject code by tests/test_consts_pin.py), so this driver never loads the
CUDA library: only the scene description and the per-frame inputs (numpy) are shared with it.
"""
from __future__ import annotations

import time

import numpy as np

from . import OracleHair, STAGE_FOLLOW, STAGE_INTEGRATE, STAGE_LENGTH_WIND, STAGE_LOCAL_SHAPE, STAGE_STRAND_LEVEL, \
    STAGE_VSP, SimParams, fill_sim_params, mesh_skin, sdf_build, sdf_collide, settings


class OracleConstants:
    """The host half of TressFXHairObject (TressFXHairObject.h:104, 129; TressFXHairObject.cpp:157,
    366-437): two constant blocks used alternately by frame parity, the frame counter, the reset flag
    and the CPU local-shape iteration count."""

    def __init__(self, n: int, F: int):
        self.n, self.F = n, F
        self.blocks = [SimParams(), SimParams()]
        self.frame = 0
        self.cpu_local_iterations = 0
        self.blocks[0].set_reset(1.0)   # the constructor's ResetPositions

    def update_simulation_parameters(self, overrides: dict, dt: float) -> None:
        self.cpu_local_iterations = fill_sim_params(self.blocks[self.frame % 2], settings(**overrides), dt, self.n,
                                                    self.F, self.frame)

    def update_bone_matrices(self, mats: np.ndarray) -> None:
        mats = np.ascontiguousarray(mats, dtype=np.float32).reshape(-1, 16)
        k = min(len(mats), 512)
        self.blocks[self.frame % 2].bones_view()[:k] = mats[:k]

    def increase_simulation_frame(self) -> None:
        self.blocks[self.frame % 2].set_reset(0.0)
        self.frame += 1

    def current_params(self) -> SimParams:
        return self.blocks[self.frame % 2]


def margin_world(obj, grid) -> float:
    """collisionMargin * cellSize in float (TressFXSDFCollision.cpp:194)."""
    return float(np.float32(obj.collision_margin_cells) * np.float32(grid.cell_size))


class OraclePipeline:
    def __init__(self, scene, dtype=np.float32, threads: int = 0):
        self._margin_world = margin_world
        self.scene = scene
        self.dtype = np.dtype(dtype)
        self.threads = threads
        self.hair = [OracleHair(o.asset, dtype) for o in scene.objects]
        self.consts = [OracleConstants(o.asset.verts_per_strand, o.asset.follow_per_guide) for o in scene.objects]
        self.sdf_words = [None] * len(scene.objects)
        self.more_words = [[None] * len(o.more) for o in scene.objects]   # further colliders
        self.frame = 0
        self.stage_seconds: dict[str, float] = {}

    def _t(self, name: str, t0: float) -> float:
        t1 = time.perf_counter()
        self.stage_seconds[name] = self.stage_seconds.get(name, 0.0) + (t1 - t0)
        return t1

    def step(self, fin) -> None:
        sc = self.scene
        for i, (h, c) in enumerate(zip(self.hair, self.consts)):
            c.update_simulation_parameters(fin.settings_overrides[i], sc.dt)
            c.update_bone_matrices(fin.hair_bones[i])
        t = time.perf_counter()
        for i, o in enumerate(sc.objects):
            if o.mesh is not None:
                skinned = mesh_skin(o.mesh.vertices, o.mesh.skinning, fin.mesh_bones[i], self.threads)
                t = self._t("BoneSkinning", t)
                self.sdf_words[i] = sdf_build(fin.grids[i], skinned, o.mesh.indices, self.dtype, self.threads)
                t = self._t("SDFBuild", t)
            for k, c in enumerate(o.more):
                skinned = mesh_skin(c.mesh.vertices, c.mesh.skinning, fin.more_bones[i][k], self.threads)
                self.more_words[i][k] = sdf_build(fin.more_grids[i][k], skinned, c.mesh.indices, self.dtype, self.threads)
                t = self._t("SDFBuild", t)
        order = [(STAGE_INTEGRATE, "IntegrationAndGlobalShapeConstraints"), (STAGE_STRAND_LEVEL, "CalculateStrandLevelData"),
                 (STAGE_VSP, "VelocityShockPropagation"), (STAGE_LOCAL_SHAPE, "LocalShapeConstraints"),
                 (STAGE_LENGTH_WIND, "LengthConstriantsWindAndCollision"), (STAGE_FOLLOW, "UpdateFollowHairVertices")]
        for st, name in order:
            for h, c in zip(self.hair, self.consts):
                reps = c.cpu_local_iterations if st == STAGE_LOCAL_SHAPE else 1
                for _ in range(reps):
                    h.stage(st, c.current_params(), self.threads)
            t = self._t(name, t)
        for c in self.consts:
            c.increase_simulation_frame()
        for i, (h, o) in enumerate(zip(self.hair, sc.objects)):
            if o.mesh is not None:
                g = fin.grids[i]
                sdf_collide(g, self.sdf_words[i], self._margin_world(o, g), h, self.threads)
            for k, c in enumerate(o.more):   # Simulation::RunCollision: every collision mesh, in order
                g = fin.more_grids[i][k]
                sdf_collide(g, self.more_words[i][k], self._margin_world(c, g), h, self.threads)
        self._t("CollideHairVerticesWithSdf", t)
        self.frame += 1
