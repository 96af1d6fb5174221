"""Oracle frame driver (test infrastructure): the sample's per-frame order on the CPU.

Mirrors tressfx_gb300.headless.PlainPipeline step for step -- skin meshes, rebuild SDFs,
simulate (stage-major over objects), collide -- with every kernel replaced by the oracle's
restatement.  Constant blocks come from the same host code (tressfx_gb300.api.SimConstants), so
the GPU and the oracle consume identical inputs.
"""
from __future__ import annotations

import time

import numpy as np

from . import OracleHair, STAGE_FOLLOW, STAGE_INTEGRATE, STAGE_LENGTH_WIND, STAGE_LOCAL_SHAPE, STAGE_STRAND_LEVEL, \
    STAGE_VSP, mesh_skin, sdf_build, sdf_collide


class OraclePipeline:
    def __init__(self, scene, dtype=np.float32, threads: int = 0):
        from tressfx_gb300.api import SimConstants
        from tressfx_gb300.synthetic import margin_world
        self._margin_world = margin_world
        self.scene = scene
        self.dtype = np.dtype(dtype)
        self.threads = threads
        self.hair = [OracleHair(o.asset, dtype) for o in scene.objects]
        self.consts = [SimConstants(o.asset.verts_per_strand, o.asset.follow_per_guide) for o in scene.objects]
        self.sdf_words = [None] * len(scene.objects)
        self.frame = 0
        self.stage_seconds: dict[str, float] = {}

    def _t(self, name: str, t0: float) -> float:
        t1 = time.perf_counter()
        self.stage_seconds[name] = self.stage_seconds.get(name, 0.0) + (t1 - t0)
        return t1

    def step(self, fin) -> None:
        sc = self.scene
        for i, (h, c) in enumerate(zip(self.hair, self.consts)):
            c.update_simulation_parameters(fin.settings[i], sc.dt)
            c.update_bone_matrices(fin.hair_bones[i])
        t = time.perf_counter()
        for i, o in enumerate(sc.objects):
            if o.mesh is not None:
                skinned = mesh_skin(o.mesh.vertices, o.mesh.skinning, fin.mesh_bones[i], self.threads)
                t = self._t("BoneSkinning", t)
                self.sdf_words[i] = sdf_build(fin.grids[i], skinned, o.mesh.indices, self.dtype, self.threads)
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
        self._t("CollideHairVerticesWithSdf", t)
        self.frame += 1
