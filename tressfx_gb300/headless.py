"""Headless frame driver: the sample's per-frame order without a window.

Simulation::StartSimulation (src/Simulation.cpp:50-94) runs, per frame:
  1. skin every collision mesh (TressFXBoneSkinning::Update),
  2. rebuild every SDF (TressFXSDFCollision::Update: Initialize, Construct, Finalize),
  3. TressFXSimulation::Simulate over all hair objects (after UpdateBones),
  4. collide every hair object with every SDF (TressFXSDFCollision::CollideWithHair).
Before that, TressFXSample::UpdateSimulationParameters (src/TressFXSample.cpp:189-195) fills each
object's constant block.  ``PlainPipeline`` issues exactly that sequence through the C ABI, one
launch per object per stage.
"""
from __future__ import annotations

import numpy as np

from . import _capi as A
from .api import CollisionMesh, Context, HairObject, SDFCollision, Simulation, default_settings
from .synthetic import Scene, SceneObject, margin_world, sdf_grid_for, wind_magnitude


def settings_struct(d: dict) -> A.SimSettings:
    s = default_settings()
    for k, v in d.items():
        if k == "wind_direction":
            for i in range(3):
                s.wind_direction[i] = float(v[i])
        else:
            setattr(s, k, v)
    return s


class FrameInputs:
    """Everything the host feeds one frame: per-object settings, hair bones, mesh bones, SDF grid.

    `settings_overrides` holds each object's settings as a dict of TressFXSimulationSettings fields
    (the scene's values with this frame's wind magnitude); `settings` turns them into the library's
    structs on first use, so that a CPU-only consumer never loads the library."""

    def __init__(self, scene: Scene, frame: int):
        t = frame * scene.dt
        self.frame = frame
        self.settings_overrides: list[dict] = []
        self._settings: list[A.SimSettings] | None = None
        self.hair_bones = []
        self.mesh_bones = []
        self.grids = []
        self.more_bones: list[list] = []   # per object: the bones and grids of its further colliders
        self.more_grids: list[list] = []
        for o in scene.objects:
            st = dict(o.settings)
            st["wind_magnitude"] = wind_magnitude(scene, o, frame)
            self.settings_overrides.append(st)
            self.hair_bones.append(o.bone_fn(t) if o.bone_fn is not None else np.eye(4, dtype=np.float32).reshape(1, 16))
            if o.mesh is not None:
                mb = o.mesh_bone_fn(t)
                self.mesh_bones.append(mb)
                self.grids.append(sdf_grid_for(o, mb))
            else:
                self.mesh_bones.append(None)
                self.grids.append(None)
            mbs = [c.mesh_bone_fn(t) for c in o.more]
            self.more_bones.append(mbs)
            self.more_grids.append([sdf_grid_for(c, mb) for c, mb in zip(o.more, mbs)])

    @property
    def settings(self) -> list[A.SimSettings]:
        if self._settings is None:
            self._settings = [settings_struct(d) for d in self.settings_overrides]
        return self._settings


class PlainPipeline:
    """All objects of a scene on the plain path of one context."""

    def __init__(self, ctx: Context, scene: Scene):
        self.ctx = ctx
        self.scene = scene
        self.hair: list[HairObject] = []
        self.meshes: list[CollisionMesh | None] = []
        self.sdfs: list[SDFCollision | None] = []
        self.sim = Simulation()
        self.frame = 0
        for o in scene.objects:
            self.hair.append(HairObject(ctx, o.asset))
            if o.mesh is not None:
                m = CollisionMesh(ctx, o.mesh.vertices, o.mesh.indices, o.mesh.skinning)
                s = SDFCollision(ctx, int(np.prod(o.sdf_dims)))
                s.bind_mesh(m)
                self.meshes.append(m)
                self.sdfs.append(s)
            else:
                self.meshes.append(None)
                self.sdfs.append(None)
        # further colliders: (mesh, sdf) per object, in collision order
        self.more: list[list[tuple[CollisionMesh, SDFCollision]]] = []
        for o in scene.objects:
            pairs = []
            for c in o.more:
                m = CollisionMesh(ctx, c.mesh.vertices, c.mesh.indices, c.mesh.skinning)
                s = SDFCollision(ctx, int(np.prod(c.sdf_dims)))
                s.bind_mesh(m)
                pairs.append((m, s))
            self.more.append(pairs)

    def prepare(self, fin: FrameInputs) -> None:
        """Host side of a frame: UpdateSimulationParameters + UpdateBones for every object."""
        for h, st, hb in zip(self.hair, fin.settings, fin.hair_bones):
            h.update_simulation_parameters(st, self.scene.dt)
            h.update_bone_matrices(hb)

    def run(self, fin: FrameInputs) -> None:
        """Device side of a frame, stream ordered (skin, SDF, simulate, collide)."""
        for m, s, mb, g in zip(self.meshes, self.sdfs, fin.mesh_bones, fin.grids):
            if m is not None:
                m.skin(mb)
                s.update(g)
        for pairs, mbs, gs in zip(self.more, fin.more_bones, fin.more_grids):
            for (m, s), mb, g in zip(pairs, mbs, gs):
                m.skin(mb)
                s.update(g)
        self.sim.simulate(self.hair)
        # Simulation::RunCollision: every collision mesh of an object, in order
        for h, s, o, g, pairs, gs in zip(self.hair, self.sdfs, self.scene.objects, fin.grids, self.more, fin.more_grids):
            if s is not None:
                s.collide(h, g, margin_world(o, g))
            for (_, sm), c, gm in zip(pairs, o.more, gs):
                sm.collide(h, gm, margin_world(c, gm))
        self.frame += 1

    def step(self, frame: int | None = None) -> FrameInputs:
        fin = FrameInputs(self.scene, self.frame if frame is None else frame)
        self.prepare(fin)
        self.run(fin)
        return fin

    def close(self) -> None:
        for x in self.hair + self.meshes + self.sdfs + [x for pairs in self.more for pair in pairs for x in pair]:
            if x is not None:
                x.close()


class BatchedPipeline(PlainPipeline):
    """The same objects as PlainPipeline, advanced by the batched path: one graph launch per frame."""

    def __init__(self, ctx: Context, scene: Scene, autotune_frames: int = 0):
        from .api import Batch
        super().__init__(ctx, scene)
        self.batch = Batch(ctx)
        self.sdf_index: list[int] = []
        for m, s, o in zip(self.meshes, self.sdfs, scene.objects):
            self.sdf_index.append(self.batch.add_sdf(s, m, o.sdf_dims) if s is not None else -1)
        self.more_index: list[list[int]] = []
        for pairs, o in zip(self.more, scene.objects):
            self.more_index.append([self.batch.add_sdf(s, m, c.sdf_dims) for (m, s), c in zip(pairs, o.more)])
        for i, (h, si) in enumerate(zip(self.hair, self.sdf_index)):
            self.batch.add_hair(h, si)
            for sj in self.more_index[i]:
                self.batch.add_hair_collision(i, sj)
        self.batch.build()
        self.autotune_frames = autotune_frames
        self._tuned = autotune_frames <= 0

    def set_inputs(self, fin: FrameInputs) -> None:
        """Host side of a frame for the batch: constants, grids and mesh bones into the frame block."""
        self.prepare(fin)
        for i, h in enumerate(self.hair):
            self.batch.set_hair_constants(i, h.current_params(), h.num_bones, h.cpu_local_iterations)
        for i, (o, si, g, mb) in enumerate(zip(self.scene.objects, self.sdf_index, fin.grids, fin.mesh_bones)):
            if si >= 0:
                self.batch.set_sdf_frame(si, g, margin_world(o, g))
                self.batch.set_mesh_bones(si, mb)
            for sj, c, gm, mbm in zip(self.more_index[i], o.more, fin.more_grids[i], fin.more_bones[i]):
                self.batch.set_sdf_frame(sj, gm, margin_world(c, gm))
                self.batch.set_mesh_bones(sj, mbm)

    def run(self, fin: FrameInputs) -> None:
        if not self._tuned:
            self.batch.autotune(self.autotune_frames)
            self._tuned = True
        self.batch.run()
        for h in self.hair:
            h.increase_simulation_frame()
        self.frame += 1

    def step(self, frame: int | None = None) -> FrameInputs:
        fin = FrameInputs(self.scene, self.frame if frame is None else frame)
        self.set_inputs(fin)
        self.run(fin)
        return fin

    def close(self) -> None:
        self.batch.close()
        super().close()


class NeuralPipeline(PlainPipeline):
    """The plain path with the learned collision proxy in front of the grid: per frame the mesh is
    skinned, the hair simulated, and tfx_nsdf_collide classifies every vertex with the network and
    collides the contact band exactly on a grid built at the band's cells only."""

    def __init__(self, ctx: Context, scene: Scene, proxy):
        super().__init__(ctx, scene)
        self.proxy = proxy
        self.band_counts: list[int] = []

    def run(self, fin: FrameInputs, record_band: bool = False) -> None:
        for m, mb in zip(self.meshes, fin.mesh_bones):
            if m is not None:
                m.skin(mb)
        self.sim.simulate(self.hair)
        pose = self.scene.meta["pose_fn"](fin.frame * self.scene.dt)
        for h, s, o, g in zip(self.hair, self.sdfs, self.scene.objects, fin.grids):
            if s is not None:
                n = self.proxy.collide(h, s, g, margin_world(o, g), pose, band=record_band)
                if record_band:
                    self.band_counts.append(n)
        self.frame += 1
