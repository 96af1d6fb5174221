"""A scene on the slice of the reference's shipped Ratboy asset in tests/golden/ratboy_subset.npz
(written by tests/golden/make_ratboy_golden.py from the reference's own loaders): the mohawk slice
with the sample's mohawk settings (src/TressFXSample.cpp:427-437), the body slice as its collision
mesh with an SDF sized by the reference's rule (TressFXSDFCollision.cpp:43-68: 50 cells across the
mesh's x extent, 0.8 x 50 cells of padding on every side), and 105 bones posed per frame.

The sample animates the skeleton from a glTF file; here each bone turns about a common pivot by its
own phase of a 1 Hz swing, so that strands and triangles skinned to different bones move apart."""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from tressfx_gb300.synthetic import Collider, HairAsset, Mesh, Scene, SceneObject, _settings, bone_matrix, rot_x, rot_y

FIXTURE = Path(__file__).resolve().parent / "golden" / "ratboy_subset.npz"
SDF_CELLS_X = 50          # TressFXCollisionMeshDescription of the body (src/TressFXSample.cpp:473-480)
HAND_CELLS_X, HAND_MARGIN = 32, 0.5   # and of each hand (:481-500)
PIVOT = np.array([0.0, 0.55, 0.05])


def load() -> dict:
    with np.load(FIXTURE, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def hair_asset(f: dict) -> HairAsset:
    counts = f["counts"]
    total_strands, total_verts, n, guides, _, follow = (int(x) for x in counts)
    return HairAsset(num_guide_strands=guides, verts_per_strand=n, follow_per_guide=follow,
                     positions=f["positions"].reshape(total_verts, 4).copy(),
                     tangents=f["tangents"].reshape(total_verts, 4).copy(),
                     rest_lengths=f["rest_lengths"].reshape(total_verts).copy(),
                     follow_root_offsets=f["follow_root_offsets"].reshape(total_strands, 4).copy(),
                     bone_skinning=f["bone_skinning"].reshape(total_strands, 8).copy())


def bones_fn(num_bones: int, amplitude_deg: float = 25.0, hz: float = 1.0):
    phase = 0.07 * np.arange(num_bones)

    def fn(t: float) -> np.ndarray:
        out = np.empty((num_bones, 16), np.float32)
        for b in range(num_bones):
            a = math.radians(amplitude_deg) * math.sin(2.0 * math.pi * hz * t + phase[b])
            R = rot_y(a) @ rot_x(0.4 * a)
            out[b] = bone_matrix(R, PIVOT).reshape(16)
        return out
    return fn


def grid_by_reference_rule(mesh: Mesh, cells_x: int):
    """(dims, cell, centre) as TressFXSDFCollision sizes a grid (TressFXSDFCollision.cpp:43-68)."""
    p = mesh.vertices[:, :3].astype(np.float32)
    lo, hi = p.min(0), p.max(0)
    cell = np.float32((hi[0] - lo[0]) / np.float32(cells_x))
    pad = np.float32(int(0.8 * cells_x)) * cell
    dims = tuple(int((hi[i] - lo[i] + 2 * pad) / cell) for i in range(3))
    return dims, float(cell), ((lo + hi) / 2).astype(np.float64)


def scene(frames: int = 12, margin_cells: float = 0.5, hands: bool = False) -> Scene:
    """The slice colliding with the body; with `hands`, then with each hand too, as the sample collides
    the mohawk with all three meshes (src/Simulation.cpp:106-118)."""
    f = load()
    asset = hair_asset(f)
    mesh = Mesh(vertices=f["mesh_vertices"].astype(np.float32).copy(), indices=f["mesh_indices"].astype(np.uint32).copy(),
                skinning=f["mesh_skinning"].astype(np.float32).copy())
    st = _settings(vsp_coeff=0.758, vsp_accel_threshold=1.208, local_constraint_stiffness=0.908,
                   local_constraints_iterations=3, global_constraint_stiffness=0.408, global_constraints_range=0.308,
                   length_constraints_iterations=3, damping=0.068, gravity_magnitude=0.09)
    dims, cell, centre = grid_by_reference_rule(mesh, SDF_CELLS_X)
    nb = int(f["num_bones"])
    fn = bones_fn(nb)
    obj = SceneObject(asset, st, fn, mesh, fn, dims, cell, centre, follow_bone=int(f["follow_bone"]),
                      collision_margin_cells=margin_cells)
    name = f"ratboy_slice_{asset.num_guide_strands}x{asset.verts_per_strand}_F{asset.follow_per_guide}"
    if hands:
        for side in ("left_hand", "right_hand"):
            hm = Mesh(vertices=f[f"{side}_vertices"].astype(np.float32).copy(),
                      indices=f[f"{side}_indices"].astype(np.uint32).copy(),
                      skinning=f[f"{side}_skinning"].astype(np.float32).copy())
            hd, hc, hctr = grid_by_reference_rule(hm, HAND_CELLS_X)
            obj.more.append(Collider(hm, fn, hd, hc, hctr, follow_bone=int(f[f"{side}_counts"][2]),
                                     collision_margin_cells=HAND_MARGIN))
        name += "_body_hands"
    return Scene(name, [obj], frames=frames)
