"""Writes the golden fixtures tests/golden/*.npz from the reference's own compute shaders.

Run where the reference checkout is mounted:  python tests/golden/make_golden.py
Each fixture stores the inputs of a short run and the SHA-256 digest of the simulation state after
each recorded kernel, as computed by oracle/hlsl_ref (the reference's HLSL compiled as C++,
dispatched with the reference's own group counts).  The constant block of every frame comes from
oracle/consts_ref (the reference's own UpdateSimulationParameters / SetWind, compiled here).  tests/golden_replay.py replays them on the
oracle and on the CUDA library.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from golden_replay import GOLDEN, INPUT_KEYS, STATE_KEYS, digest, state_digest  # noqa: E402


class RefBackend:
    def load(self, asset, fx):
        import oracle
        from oracle import hlsl_ref
        self.o = oracle
        self.lib = hlsl_ref.lib()
        self.h = oracle.OracleHair(asset)
        self.fx = fx

    def set_constants(self, p, nb):
        self.p = p

    def stage(self, k):
        if self.lib.tfxr_sim_dispatch(k, C.addressof(self.h._struct), C.addressof(self.p)):
            raise RuntimeError("reference dispatch failed")

    def state(self):
        return {k: getattr(self.h, k) for k in STATE_KEYS}

    def mesh_skin(self, bones):
        v = np.ascontiguousarray(self.fx["mesh_vertices"], dtype=np.float32)
        out = v.copy()
        full = np.zeros((512, 16), dtype=np.float32)
        b = np.asarray(bones, dtype=np.float32).reshape(-1, 16)
        full[:len(b)] = b
        sk = np.ascontiguousarray(self.fx["mesh_skinning"], dtype=np.float32)
        self.lib.tfxr_mesh_skin(out.ctypes.data, v.ctypes.data, sk.ctypes.data, full.ctypes.data, len(v))
        self.skinned = out
        return out

    def _alloc(self, g):
        return max(int(np.float32(1.4) * np.float32(g.num_cells)), g.num_cells)

    def sdf_build(self, g):
        words = np.zeros(self._alloc(g), dtype=np.uint32)
        gp = self.o.sdf_params(g)
        idx = np.ascontiguousarray(self.fx["mesh_indices"], dtype=np.uint32)
        self.lib.tfxr_sdf_update(words.ctypes.data, len(words), C.addressof(gp), self.skinned.ctypes.data,
                                 len(self.skinned), idx.ctypes.data, len(idx) // 3)
        self.words = words
        return words[:g.num_cells].copy()

    def collide(self, g, margin):
        gp = self.o.sdf_params(g)
        self.lib.tfxr_sdf_collide(self.words.ctypes.data, len(self.words), C.addressof(gp), margin,
                                  C.addressof(self.h._struct))


def cases():
    from tressfx_gb300 import synthetic as S
    small16 = S.scene_small(seed=101, num_guides=64, n=16)
    small4 = S.scene_small(seed=102, num_guides=64, n=4)
    small64 = S.scene_small(seed=103, num_guides=64, n=64)
    small64.objects[0].settings.update(local_constraints_iterations=3, wind_magnitude=3.0, length_constraints_iterations=2)
    small32 = S.scene_small(seed=105, num_guides=128, n=32)
    small32.objects[0].settings.update(local_constraints_iterations=2, wind_magnitude=1.0, tip_separation=0.5)
    head = S.scene_head(seed=104, num_guides=64, n=8, follows=1, triangles=1200, sdf_cells=20, frames=4)
    # the slice of the shipped Ratboy asset (tests/golden/ratboy_subset.npz): its arrays stay in that file
    import ratboy_scene
    ratboy = ratboy_scene.scene(frames=5, margin_cells=0.5)
    ratboy.meta["inputs_from"] = "ratboy_subset"
    return [("small_64x16", small16, 5, {2}), ("small_64x4", small4, 6, {2, 5}), ("small_64x64_wind", small64, 3, {2}),
            ("small_128x32_wind", small32, 4, {3}), ("head_64x8_F1_sdf20", head, 4, {2, 3}),
            ("real_ratboy_slice_sdf", ratboy, 5, {2, 4})]


def make(name, scene, frames, stage_frames) -> dict:
    import oracle
    import oracle.consts_ref as R
    from tressfx_gb300.headless import FrameInputs
    from tressfx_gb300.synthetic import margin_world
    from golden_replay import Asset  # noqa: F401
    o = scene.objects[0]
    a = o.asset
    fx: dict = {"counts": np.array([a.num_guide_strands, a.verts_per_strand, a.follow_per_guide], dtype=np.int32),
                "positions": a.positions, "tangents": a.tangents, "rest_lengths": a.rest_lengths,
                "follow_root_offsets": a.follow_root_offsets, "bone_skinning": a.bone_skinning,
                "frames": np.int32(frames)}
    if o.mesh is not None:
        fx["mesh_vertices"] = o.mesh.vertices
        fx["mesh_indices"] = o.mesh.indices
        fx["mesh_skinning"] = o.mesh.skinning
        fx["grid_dims"] = np.array(o.sdf_dims, dtype=np.int32)

    class _A:
        pass
    asset = _A()
    asset.num_guide_strands, asset.verts_per_strand, asset.follow_per_guide = a.num_guide_strands, a.verts_per_strand, a.follow_per_guide
    asset.positions, asset.tangents, asset.rest_lengths = a.positions, a.tangents, a.rest_lengths
    asset.follow_root_offsets, asset.bone_skinning = a.follow_root_offsets, a.bone_skinning
    ref = RefBackend()
    ref.load(asset, fx)
    # the constant block of every frame from the reference's own UpdateSimulationParameters / SetWind
    blocks = [oracle.SimParams(), oracle.SimParams()]
    for f in range(frames):
        fin = FrameInputs(scene, f)
        hdr, cpu_iters = R.update_simulation_parameters(R.settings(**fin.settings_overrides[0]), scene.dt,
                                                        a.verts_per_strand, a.follow_per_guide, f)
        p = blocks[f % 2]
        C.memmove(p.header, hdr, 160)
        bones = np.ascontiguousarray(fin.hair_bones[0], dtype=np.float32).reshape(-1, 16)
        num_bones = min(len(bones), 512)
        p.bones_view()[:num_bones] = bones[:num_bones]
        fx[f"cb_header_{f}"] = np.frombuffer(hdr, dtype=np.uint8).copy()
        fx[f"cb_bones_{f}"] = p.bones_view()[:num_bones].copy()
        fx[f"cpu_iters_{f}"] = np.int32(cpu_iters)
        ref.set_constants(p, num_bones)
        if o.mesh is not None:
            g = fin.grids[0]
            fx[f"mesh_bones_{f}"] = np.asarray(fin.mesh_bones[0], dtype=np.float32)
            fx[f"grid_origin_{f}"] = np.array(list(g.origin), dtype=np.float32)
            fx[f"grid_cell_{f}"] = np.float32(g.cell_size)
            fx[f"margin_{f}"] = np.float32(margin_world(o, g))
            fx[f"h_skinned_{f}"] = digest(ref.mesh_skin(fx[f"mesh_bones_{f}"]))
            fx[f"h_sdf_{f}"] = digest(ref.sdf_build(g))
        for k in (1, 2, 3, 4, 5, 6):
            for _ in range(cpu_iters if k == 4 else 1):
                ref.stage(k)
            if f in stage_frames:
                fx[f"h_stage{k}_{f}"] = state_digest(ref.state())
        if o.mesh is not None:
            ref.collide(fin.grids[0], float(fx[f"margin_{f}"]))
        fx[f"h_end_{f}"] = state_digest(ref.state())
    for k in STATE_KEYS:
        fx[f"final_{k}"] = ref.state()[k].copy()
    if "inputs_from" in scene.meta:   # asset and mesh arrays are read from that fixture on replay
        for k in INPUT_KEYS + tuple(f"final_{k}" for k in STATE_KEYS):
            fx.pop(k, None)
        fx["inputs_from"] = np.array(scene.meta["inputs_from"])
    return fx


def main() -> None:
    from oracle import hlsl_ref
    if not hlsl_ref.available():
        raise SystemExit("the reference shader sources are not mounted here")
    hlsl_ref.build()
    GOLDEN.mkdir(exist_ok=True)
    for name, scene, frames, stage_frames in cases():
        fx = make(name, scene, frames, stage_frames)
        np.savez_compressed(GOLDEN / f"{name}.npz", **fx)
        print(name, (GOLDEN / f"{name}.npz").stat().st_size, "bytes")


if __name__ == "__main__":
    main()
