"""Seeded synthetic workloads: hair assets, collision meshes and skeletal animation.

The hair asset arrays follow TressFXAsset after GenerateFollowHairs + ProcessAsset
(src/TressFX/TressFXAsset.cpp:177-399): strand-major float4 positions with w = inverse mass
(vertices 0 and 1 immovable), follow strands stored right after their guide, follow root offsets
(xyz offset, w = guide strand index), tangents, rest lengths |p_j - p_{j+1}| (0 on the last
vertex), and per-strand {boneIndex.xyzw, boneWeight.xyzw}.  Bone matrices are row-major 4x4 in
the row-vector convention the shaders use (p' = [p 1] * M).

Every generator takes a seed; the same seed gives the same arrays on every platform.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


# ---------------------------------------------------------------------------------------- asset
@dataclass
class HairAsset:
    num_guide_strands: int
    verts_per_strand: int
    follow_per_guide: int
    positions: np.ndarray          # float32 [Vtot, 4]
    tangents: np.ndarray           # float32 [Vtot, 4]
    rest_lengths: np.ndarray       # float32 [Vtot]
    follow_root_offsets: np.ndarray  # float32 [Stot, 4]
    bone_skinning: np.ndarray      # float32 [Stot, 8]

    @property
    def num_strands(self) -> int:
        return self.num_guide_strands * (self.follow_per_guide + 1)

    @property
    def num_vertices(self) -> int:
        return self.num_strands * self.verts_per_strand


def _normalize(v: np.ndarray) -> np.ndarray:
    n = np.linalg.norm(v, axis=-1, keepdims=True)
    return v / np.maximum(n, 1e-30)


def _perpendicular_frame(d: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    a = np.where(np.abs(d[:, :1]) < 0.9, np.array([[1.0, 0.0, 0.0]]), np.array([[0.0, 1.0, 0.0]]))
    t0 = _normalize(np.cross(d, a))
    t1 = np.cross(d, t0)
    return t0, t1


def grow_strands(roots: np.ndarray, normals: np.ndarray, n: int, segment: float, turn_deg: float,
                 rng: np.random.Generator, droop: float = 0.35) -> np.ndarray:
    """Smoothed random walks: each step turns the heading by ~N(0, turn_deg) about a random
    perpendicular axis, blended with a gentle pull toward -y. Returns float64 [G, n, 3]."""
    G = len(roots)
    out = np.empty((G, n, 3))
    out[:, 0] = roots
    d = _normalize(normals.astype(np.float64))
    turn = math.radians(turn_deg)
    for j in range(1, n):
        ang = rng.normal(0.0, turn, size=(G, 1))
        phi = rng.uniform(0.0, 2.0 * math.pi, size=(G, 1))
        t0, t1 = _perpendicular_frame(d)
        axis_dir = np.cos(phi) * t0 + np.sin(phi) * t1
        d = _normalize(np.cos(ang) * d + np.sin(ang) * axis_dir)
        d = _normalize(d + droop * (j / n) * np.array([[0.0, -1.0, 0.0]]) * 0.3)
        out[:, j] = out[:, j - 1] + segment * d
    return out


def _tangent_vectors(n: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """GetTangentVectors, TressFXAsset.cpp:37-63 (float32)."""
    n = n.astype(np.float32)
    t0 = np.zeros_like(n)
    t1 = np.zeros_like(n)
    big_z = np.abs(n[:, 2]) > np.float32(0.707)
    a = n[:, 1] * n[:, 1] + n[:, 2] * n[:, 2]
    k = np.float32(1.0) / np.sqrt(a)
    t0[big_z, 1] = -n[big_z, 2] * k[big_z]
    t0[big_z, 2] = n[big_z, 1] * k[big_z]
    t1[big_z, 0] = a[big_z] * k[big_z]
    t1[big_z, 1] = -n[big_z, 0] * t0[big_z, 2]
    t1[big_z, 2] = n[big_z, 0] * t0[big_z, 1]
    s = ~big_z
    a2 = n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]
    k2 = np.float32(1.0) / np.sqrt(a2)
    t0[s, 0] = -n[s, 1] * k2[s]
    t0[s, 1] = n[s, 0] * k2[s]
    t1[s, 0] = -n[s, 2] * t0[s, 1]
    t1[s, 1] = n[s, 2] * t0[s, 0]
    t1[s, 2] = a2[s] * k2[s]
    return t0, t1


def build_asset(guides: np.ndarray, follow_per_guide: int = 0, tip_separation: float = 0.0,
                follow_radius: float = 0.0, rng: np.random.Generator | None = None,
                bone_skinning: np.ndarray | None = None) -> HairAsset:
    """Guide polylines [G, n, 3] -> a processed asset (GenerateFollowHairs + ProcessAsset)."""
    G, n, _ = guides.shape
    F = follow_per_guide
    S = G * (F + 1)
    pos = np.zeros((S, n, 4), dtype=np.float32)
    g32 = guides.astype(np.float32)
    w = np.ones(n, dtype=np.float32)
    w[:2] = 0.0
    gidx = np.arange(G) * (F + 1)
    pos[gidx, :, :3] = g32
    pos[gidx, :, 3] = w
    offsets = np.zeros((S, 4), dtype=np.float32)
    offsets[gidx, 3] = gidx.astype(np.float32)
    if F > 0:
        rng = rng if rng is not None else np.random.default_rng(0)
        v01 = g32[:, 1] - g32[:, 0]
        v01 = v01 / np.sqrt((v01 * v01).sum(axis=1, keepdims=True))
        t0, t1 = _tangent_vectors(v01)
        factor = (np.float32(tip_separation) * (np.arange(n, dtype=np.float32) / np.float32(n)) + np.float32(1.0))
        for i in range(F):
            r0 = rng.uniform(-follow_radius, follow_radius, size=(G, 1)).astype(np.float32)
            r1 = rng.uniform(-follow_radius, follow_radius, size=(G, 1)).astype(np.float32)
            off = r0 * t0 + r1 * t1
            fi = gidx + i + 1
            offsets[fi, :3] = off
            offsets[fi, 3] = gidx.astype(np.float32)
            pos[fi, :, :3] = g32 + off[:, None, :] * factor[None, :, None]
            pos[fi, :, 3] = w
    # ComputeStrandTangent (TressFXAsset.cpp:304-342), float32
    p3 = pos[:, :, :3]
    tan = np.zeros((S, n, 4), dtype=np.float32)
    d0 = p3[:, 1] - p3[:, 0]
    tan[:, 0, :3] = d0 / np.sqrt((d0 * d0).sum(-1, keepdims=True))
    pre = p3[:, 1:-1] - p3[:, :-2]
    nxt = p3[:, 2:] - p3[:, 1:-1]
    pre = pre / np.sqrt((pre * pre).sum(-1, keepdims=True))
    nxt = nxt / np.sqrt((nxt * nxt).sum(-1, keepdims=True))
    t = pre + nxt
    tan[:, 1:-1, :3] = t / np.sqrt((t * t).sum(-1, keepdims=True))
    # ComputeRestLengths (TressFXAsset.cpp:377-399)
    seg = p3[:, :-1] - p3[:, 1:]
    rest = np.zeros((S, n), dtype=np.float32)
    rest[:, :-1] = np.sqrt(seg[..., 0] * seg[..., 0] + seg[..., 1] * seg[..., 1] + seg[..., 2] * seg[..., 2])
    skin = np.zeros((S, 8), dtype=np.float32)
    if bone_skinning is None:
        skin[gidx, 4] = 1.0
    else:
        skin[gidx] = bone_skinning
    return HairAsset(G, n, F, pos.reshape(-1, 4), tan.reshape(-1, 4), rest.reshape(-1), offsets, skin)


# ---------------------------------------------------------------------------------------- bones
def rot_x(a: float) -> np.ndarray:
    c, s = math.cos(a), math.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def rot_y(a: float) -> np.ndarray:
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def rot_z(a: float) -> np.ndarray:
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])


def bone_matrix(R: np.ndarray, pivot=(0.0, 0.0, 0.0), translation=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Row-vector 4x4 for p' = R (p - pivot) + pivot + translation, flattened row-major (16 float32)."""
    M = np.eye(4)
    M[:3, :3] = R.T
    c = np.asarray(pivot, dtype=np.float64)
    M[3, :3] = c - c @ R.T + np.asarray(translation, dtype=np.float64)
    return M.astype(np.float32).reshape(16)


# ---------------------------------------------------------------------------------------- meshes
@dataclass
class Mesh:
    vertices: np.ndarray   # float32 [V, 8] = position.xyzw, normal.xyzw
    indices: np.ndarray    # uint32 [3T]
    skinning: np.ndarray   # float32 [V, 8]

    @property
    def num_triangles(self) -> int:
        return len(self.indices) // 3


def ellipsoid_mesh(center, radii, n_lat: int, n_lon: int) -> tuple[np.ndarray, np.ndarray]:
    """UV ellipsoid: returns (vertices [V, 8] float32, indices uint32), outward winding."""
    lat = np.linspace(0.0, math.pi, n_lat + 1)
    lon = np.linspace(0.0, 2.0 * math.pi, n_lon, endpoint=False)
    th, ph = np.meshgrid(lat[1:-1], lon, indexing="ij")
    unit = np.stack([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)], axis=-1).reshape(-1, 3)
    unit = np.concatenate([[[0.0, 1.0, 0.0]], unit, [[0.0, -1.0, 0.0]]], axis=0)
    r = np.asarray(radii, dtype=np.float64)
    p = unit * r + np.asarray(center, dtype=np.float64)
    nrm = _normalize(unit / r)
    V = len(p)
    tris = []
    ring = lambda i: 1 + i * n_lon  # noqa: E731
    for k in range(n_lon):  # top cap
        tris.append((0, ring(0) + (k + 1) % n_lon, ring(0) + k))
    for i in range(n_lat - 2):
        for k in range(n_lon):
            a, b = ring(i) + k, ring(i) + (k + 1) % n_lon
            c, d = ring(i + 1) + k, ring(i + 1) + (k + 1) % n_lon
            tris.append((a, b, d))
            tris.append((a, d, c))
    last = V - 1
    for k in range(n_lon):
        tris.append((last, ring(n_lat - 2) + k, ring(n_lat - 2) + (k + 1) % n_lon))
    verts = np.zeros((V, 8), dtype=np.float32)
    verts[:, :3] = p
    verts[:, 3] = 1.0
    verts[:, 4:7] = nrm
    idx = np.asarray(tris, dtype=np.uint32).reshape(-1)
    # make every triangle's geometric normal point outward: (x1-x0) x (x2-x0) . (x0-center) > 0
    t = idx.reshape(-1, 3)
    x0, x1, x2 = p[t[:, 0]], p[t[:, 1]], p[t[:, 2]]
    flip = (np.cross(x1 - x0, x2 - x0) * (x0 - np.asarray(center))).sum(-1) < 0
    t[flip] = t[flip][:, [0, 2, 1]]
    return verts, t.reshape(-1).astype(np.uint32)


def merge_meshes(parts: list[tuple[np.ndarray, np.ndarray, np.ndarray]]) -> Mesh:
    vs, ids, sks = [], [], []
    base = 0
    for v, i, s in parts:
        vs.append(v)
        ids.append(i + base)
        sks.append(s)
        base += len(v)
    return Mesh(np.concatenate(vs), np.concatenate(ids).astype(np.uint32), np.concatenate(sks))


def mesh_lat_lon_for(tris: int) -> tuple[int, int]:
    """(n_lat, n_lon) of a UV ellipsoid with about `tris` triangles (2*n_lon*(n_lat-1))."""
    n_lon = max(8, int(round(math.sqrt(tris))))
    n_lat = max(3, int(round(tris / (2 * n_lon))) + 1)
    return n_lat, n_lon


def sample_on_ellipsoid(center, radii, count: int, rng: np.random.Generator, y_min: float = -1.0):
    """Points uniform in direction over the part of the unit sphere with y >= y_min, mapped to the
    ellipsoid; returns (points, outward normals) float64."""
    out = []
    need = count
    while need > 0:
        u = rng.normal(size=(need * 2 + 16, 3))
        u = _normalize(u)
        u = u[u[:, 1] >= y_min]
        out.append(u[:need])
        need -= len(out[-1])
    u = np.concatenate(out)[:count]
    r = np.asarray(radii, dtype=np.float64)
    return u * r + np.asarray(center, dtype=np.float64), _normalize(u / r)


# ---------------------------------------------------------------------------------------- scenes
@dataclass
class Collider:
    """A further collision mesh of a hair object, collided after the object's first (SceneObject.mesh) and
    its earlier further meshes: Simulation::RunCollision applies every collision mesh to every hair
    object in turn (src/Simulation.cpp:106-118).  Same fields as the object's own mesh."""
    mesh: Mesh
    mesh_bone_fn: object
    sdf_dims: tuple[int, int, int]
    sdf_cell: float
    sdf_center0: np.ndarray
    follow_bone: int = 0
    collision_margin_cells: float = 0.5


@dataclass
class SceneObject:
    asset: HairAsset
    settings: dict
    bone_fn: object = None            # t -> [nb, 16] float32 hair bone matrices
    mesh: Mesh | None = None
    mesh_bone_fn: object = None       # t -> [nb, 16] mesh bone matrices
    sdf_dims: tuple[int, int, int] | None = None
    sdf_cell: float = 0.0
    sdf_center0: np.ndarray | None = None   # initial grid centre
    follow_bone: int = 0              # bone whose motion moves the grid (TressFXBoneSkinning::GetBoundingBox)
    collision_margin_cells: float = 0.5
    more: list = field(default_factory=list)   # further Colliders, in collision order (needs `mesh`)


@dataclass
class Scene:
    name: str
    objects: list[SceneObject]
    dt: float = 1.0 / 60.0
    frames: int = 120
    meta: dict = field(default_factory=dict)

    @property
    def vertices_per_frame(self) -> int:
        return sum(o.asset.num_vertices for o in self.objects)


def _settings(**kw) -> dict:
    base = dict(vsp_coeff=0.8, vsp_accel_threshold=1.4, local_constraint_stiffness=0.9, local_constraints_iterations=2,
                global_constraint_stiffness=0.0, global_constraints_range=0.0, length_constraints_iterations=2,
                damping=0.08, gravity_magnitude=0.0, tip_separation=0.0, wind_magnitude=0.0,
                wind_direction=(1.0, 0.0, 0.0))
    base.update(kw)
    return base


def rigid_oscillation_bones(amplitude_deg: float = 30.0, hz: float = 1.0, axis: str = "y"):
    rot = {"x": rot_x, "y": rot_y, "z": rot_z}[axis]

    def fn(t: float) -> np.ndarray:
        a = math.radians(amplitude_deg) * math.sin(2.0 * math.pi * hz * t)
        return bone_matrix(rot(a))[None, :]
    return fn


def nod_turn_bones(pivot, nod_deg=20.0, turn_deg=30.0, nod_hz=0.7, turn_hz=0.45):
    """3 joints: 0 = neck base (static), 1 = nod about x at the pivot, 2 = turn about y after the nod."""
    def fn(t: float) -> np.ndarray:
        a = math.radians(nod_deg) * math.sin(2.0 * math.pi * nod_hz * t)
        b = math.radians(turn_deg) * math.sin(2.0 * math.pi * turn_hz * t)
        R1 = rot_x(a)
        R2 = rot_y(b) @ R1
        return np.stack([bone_matrix(np.eye(3), pivot), bone_matrix(R1, pivot), bone_matrix(R2, pivot)])
    return fn


def pose_bones(pivot, angles) -> np.ndarray:
    """3-joint pose (neck tilt about z, nod about x, turn about y) in radians -> [3, 16]."""
    a, b, c = angles
    R0 = rot_z(a)
    R1 = R0 @ rot_x(b)
    R2 = rot_y(c) @ R1
    return np.stack([bone_matrix(R0, pivot), bone_matrix(R1, pivot), bone_matrix(R2, pivot)])


def scene_small(seed: int = 1, num_guides: int = 2048, n: int = 16) -> Scene:
    """One object, guides on a 0.1 m sphere, 8 mm segments, N(0, 15 deg) turns, rigid +-30 deg at 1 Hz,
    dt 1/60, damping 0.035, global 0.2 / range 0.3, local 0.8, 1 local + 1 length iteration,
    VSP 0.5, gravity 9.8, no wind, no follow hairs, no SDF."""
    rng = np.random.default_rng(seed)
    roots, normals = sample_on_ellipsoid((0.0, 0.0, 0.0), (0.1, 0.1, 0.1), num_guides, rng)
    guides = grow_strands(roots, normals, n, 0.008, 15.0, rng)
    asset = build_asset(guides)
    st = _settings(damping=0.035, global_constraint_stiffness=0.2, global_constraints_range=0.3,
                   local_constraint_stiffness=0.8, local_constraints_iterations=1, length_constraints_iterations=1,
                   vsp_coeff=0.5, gravity_magnitude=9.8)
    return Scene("plain_small_2048x16", [SceneObject(asset, st, rigid_oscillation_bones(30.0, 1.0, "y"))], frames=120)


HEAD_CENTER = (0.0, 1.6, 0.0)
NECK_PIVOT = (0.0, 1.48, 0.0)


def head_mesh(triangles: int) -> Mesh:
    """Sphere head (r 0.1 m) + ellipsoid jaw/neck, ~`triangles` triangles, 3-joint skinning."""
    nl, nq = mesh_lat_lon_for(int(triangles * 0.7))
    hv, hi = ellipsoid_mesh(HEAD_CENTER, (0.1, 0.1, 0.1), nl, nq)
    nl2, nq2 = mesh_lat_lon_for(int(triangles * 0.3))
    ev, ei = ellipsoid_mesh((0.0, 1.5, 0.015), (0.06, 0.09, 0.07), nl2, nq2)
    hs = np.zeros((len(hv), 8), dtype=np.float32)
    hs[:, 0:4] = (2, 1, 0, 0)
    hs[:, 4:8] = (1, 0, 0, 0)
    # jaw/neck: blend nod-joint / base by height
    es = np.zeros((len(ev), 8), dtype=np.float32)
    wgt = np.clip((ev[:, 1] - 1.42) / 0.16, 0.0, 1.0)
    es[:, 0:4] = (1, 0, 0, 0)
    es[:, 4] = wgt
    es[:, 5] = 1.0 - wgt
    es[wgt <= 0.0, 4] = 1.0
    es[wgt <= 0.0, 0] = 0
    return merge_meshes([(hv, hi, hs), (ev, ei, es)])


def scene_head(seed: int = 2, num_guides: int = 20000, n: int = 32, follows: int = 4, triangles: int = 20000,
               sdf_cells: int = 64, frames: int = 300) -> Scene:
    """Full per-frame pipeline: guides on the head sphere, 4 follows (+-2 mm), 3-joint nod/turn,
    SDF 64^3 with a 2 cm margin rebuilt every frame, 3 local + 3 length iterations, VSP on,
    wind 2 m/s with +-30 % per-frame noise."""
    rng = np.random.default_rng(seed)
    roots, normals = sample_on_ellipsoid(HEAD_CENTER, (0.1, 0.1, 0.1), num_guides, rng, y_min=-0.2)
    guides = grow_strands(roots, normals, n, 0.005, 15.0, rng)
    skin = np.zeros((num_guides, 8), dtype=np.float32)
    skin[:, 0:4] = (2, 0, 0, 0)
    skin[:, 4:8] = (1, 0, 0, 0)
    asset = build_asset(guides, follows, tip_separation=1.0, follow_radius=0.002, rng=rng, bone_skinning=skin)
    st = _settings(local_constraints_iterations=3, length_constraints_iterations=3, vsp_coeff=0.758,
                   vsp_accel_threshold=1.208, local_constraint_stiffness=0.908, global_constraint_stiffness=0.408,
                   global_constraints_range=0.308, damping=0.068, gravity_magnitude=9.8, tip_separation=1.0,
                   wind_magnitude=2.0, wind_direction=(1.0, 0.0, 0.3))
    mesh = head_mesh(triangles)
    bones = nod_turn_bones(NECK_PIVOT)
    p = mesh.vertices[:, :3].astype(np.float64)
    lo, hi = p.min(0), p.max(0)
    extent = float((hi - lo).max()) + 2 * 0.02
    cell = extent / sdf_cells
    obj = SceneObject(asset, st, bones, mesh, bones, (sdf_cells,) * 3, cell, (lo + hi) / 2, follow_bone=2)
    sc = Scene(f"head_{num_guides}x{n}_F{follows}_sdf{sdf_cells}", [obj], frames=frames)
    sc.meta["wind_noise"] = 0.3
    sc.meta["wind_seed"] = seed + 1000
    return sc


def pose_trajectory(seed: int = 9, amplitude_deg: float = 38.0):
    """Smooth 3-joint pose (neck tilt, nod, turn) within +-amplitude: t -> angles (radians)."""
    rng = np.random.default_rng(seed)
    hz = rng.uniform(0.2, 0.6, 3)
    ph = rng.uniform(0.0, 2.0 * math.pi, 3)
    amp = math.radians(amplitude_deg)

    def fn(t: float) -> np.ndarray:
        return amp * np.sin(2.0 * math.pi * hz * t + ph)
    return fn


def scene_neural(seed: int = 9, num_guides: int = 20000, n: int = 32, triangles: int = 20000, sdf_cells: int = 128,
                 frames: int = 300) -> Scene:
    """The head scene's guides (no follow hairs) and mesh, driven by a 3-joint pose in +-40 degrees,
    with a 128^3 grid: the workload of the learned collision proxy."""
    sc = scene_head(seed=seed, num_guides=num_guides, n=n, follows=0, triangles=triangles, sdf_cells=sdf_cells,
                    frames=frames)
    traj = pose_trajectory(seed + 1)
    obj = sc.objects[0]
    bones = lambda t: pose_bones(NECK_PIVOT, traj(t))  # noqa: E731
    obj.bone_fn = bones
    obj.mesh_bone_fn = bones
    sc.meta["pose_fn"] = traj
    sc.name = f"neural_{num_guides}x{n}_sdf{sdf_cells}"
    return sc


def torso_mesh(triangles: int) -> Mesh:
    nl, nq = mesh_lat_lon_for(triangles)
    v, i = ellipsoid_mesh((0.0, 1.2, 0.0), (0.18, 0.3, 0.12), nl, nq)
    s = np.zeros((len(v), 8), dtype=np.float32)
    wgt = np.clip((v[:, 1] - 0.95) / 0.5, 0.0, 1.0)
    s[:, 0:4] = (1, 0, 0, 0)
    s[:, 4] = wgt
    s[:, 5] = 1.0 - wgt
    s[wgt <= 0.0, 0] = 0
    s[wgt <= 0.0, 4] = 1.0
    return Mesh(v, i, s)


def scene_fur(seed: int = 3, num_strands: int = 200000, n: int = 16, triangles: int = 50000, sdf_cells: int = 128,
              frames: int = 300) -> Scene:
    """Fur scale: strands uniform over a torso ellipsoid, 3 mm segments, SDF 128^3, 2 local + 2 length
    iterations, local stiffness 0.9, no follow hairs."""
    rng = np.random.default_rng(seed)
    roots, normals = sample_on_ellipsoid((0.0, 1.2, 0.0), (0.18, 0.3, 0.12), num_strands, rng)
    guides = grow_strands(roots, normals, n, 0.003, 15.0, rng, droop=0.2)
    wgt = np.clip((roots[:, 1] - 0.95) / 0.5, 0.0, 1.0).astype(np.float32)
    skin = np.zeros((num_strands, 8), dtype=np.float32)
    skin[:, 0:4] = (1, 0, 0, 0)
    skin[:, 4] = np.where(wgt > 0, wgt, 1.0)
    skin[:, 5] = np.where(wgt > 0, 1.0 - wgt, 0.0)
    skin[wgt <= 0, 0] = 0
    asset = build_asset(guides, 0, rng=rng, bone_skinning=skin)
    st = _settings(local_constraints_iterations=2, length_constraints_iterations=2, local_constraint_stiffness=0.9,
                   global_constraint_stiffness=0.3, global_constraints_range=0.5, damping=0.06, gravity_magnitude=9.8,
                   vsp_coeff=0.7)
    mesh = torso_mesh(triangles)
    bones = nod_turn_bones((0.0, 0.95, 0.0), nod_deg=10.0, turn_deg=20.0)
    p = mesh.vertices[:, :3].astype(np.float64)
    lo, hi = p.min(0), p.max(0)
    extent = float((hi - lo).max()) + 2 * 0.02
    obj = SceneObject(asset, st, bones, mesh, bones, (sdf_cells,) * 3, extent / sdf_cells, (lo + hi) / 2, follow_bone=1)
    return Scene(f"fur_{num_strands}x{n}_sdf{sdf_cells}", [obj], frames=frames)


def wind_magnitude(scene: Scene, obj: SceneObject, frame: int) -> float:
    """Per-frame wind magnitude: the setting x (1 + noise*U(-1,1)), seeded per frame."""
    base = obj.settings.get("wind_magnitude", 0.0)
    noise = scene.meta.get("wind_noise", 0.0)
    if base == 0.0 or noise == 0.0:
        return base
    r = np.random.default_rng([scene.meta.get("wind_seed", 0), frame]).uniform(-1.0, 1.0)
    return float(base * (1.0 + noise * r))


def margin_world(obj: SceneObject, grid) -> float:
    """collisionMargin * cellSize in float (TressFXSDFCollision.cpp:194)."""
    return float(np.float32(obj.collision_margin_cells) * np.float32(grid.cell_size))


def sdf_grid_for(obj: SceneObject, bones: np.ndarray):
    """Grid (origin, cell, dims) for a frame: the initial grid centre moved by the follow bone
    (TressFXBoneSkinning::GetBoundingBox, TressFXBoneSkinning.cpp:439-452)."""
    from ._capi import SdfGrid
    M = bones[obj.follow_bone].reshape(4, 4).astype(np.float32)
    c = obj.sdf_center0.astype(np.float32)
    nc = (np.concatenate([c, [1.0]]).astype(np.float32) @ M)[:3]
    nx, ny, nz = obj.sdf_dims
    cell = np.float32(obj.sdf_cell)
    half = np.array([nx, ny, nz], dtype=np.float32) * cell * np.float32(0.5)
    origin = (nc - half).astype(np.float32)
    g = SdfGrid()
    g.origin[0], g.origin[1], g.origin[2], g.origin[3] = float(origin[0]), float(origin[1]), float(origin[2]), 0.0
    g.cell_size = float(cell)
    g.num_cells_x, g.num_cells_y, g.num_cells_z = nx, ny, nz
    return g


def scene_batched(seed: int = 4, num_objects: int = 64, min_strands: int = 512, max_strands: int = 50000,
                  verts=(8, 16, 32, 64), min_tris: int = 5000, max_tris: int = 30000, sdf_choices=(32, 48, 64, 96, 128),
                  follows: int = 0, frames: int = 300) -> Scene:
    """Batched uneven workload: `num_objects` hair objects, strand counts log-uniform in
    [min_strands, max_strands] padded to a multiple of 64 (the reference's asset rule), vertices per
    strand drawn from `verts`, damping ~U(0.01, 0.1), stiffnesses ~U(0.1, 0.9), each object on its
    own head mesh (triangles log-uniform in [min_tris, max_tris]) with its own SDF of 32^3..128^3
    and its own nod/turn phase.  Objects sit on a 1 m grid so their SDFs do not overlap."""
    rng = np.random.default_rng(seed)
    objs = []
    side = int(math.ceil(math.sqrt(num_objects)))
    for k in range(num_objects):
        G = int(math.exp(rng.uniform(math.log(min_strands), math.log(max_strands))))
        G = max(64, ((G + 63) // 64) * 64)
        n = int(rng.choice(verts))
        tris = int(math.exp(rng.uniform(math.log(min_tris), math.log(max_tris))))
        dims = int(rng.choice(sdf_choices))
        cx, cz = (k % side) * 1.0, (k // side) * 1.0
        center = (cx, 1.6, cz)
        roots, normals = sample_on_ellipsoid(center, (0.1, 0.1, 0.1), G, rng, y_min=-0.2)
        seg = 0.12 / n
        guides = grow_strands(roots, normals, n, seg, 15.0, rng)
        skin = np.zeros((G, 8), dtype=np.float32)
        skin[:, 0:4] = (2, 0, 0, 0)
        skin[:, 4:8] = (1, 0, 0, 0)
        asset = build_asset(guides, follows, tip_separation=0.5, follow_radius=0.002, rng=rng, bone_skinning=skin)
        st = _settings(damping=float(rng.uniform(0.01, 0.1)), local_constraint_stiffness=float(rng.uniform(0.1, 0.9)),
                       global_constraint_stiffness=float(rng.uniform(0.1, 0.9)), global_constraints_range=0.3,
                       local_constraints_iterations=2, length_constraints_iterations=2, gravity_magnitude=9.8,
                       vsp_coeff=0.6, wind_magnitude=float(rng.uniform(0.0, 2.0)))
        nl, nq = mesh_lat_lon_for(int(tris * 0.7))
        hv, hi = ellipsoid_mesh(center, (0.1, 0.1, 0.1), nl, nq)
        nl2, nq2 = mesh_lat_lon_for(int(tris * 0.3))
        ev, ei = ellipsoid_mesh((cx, 1.5, cz + 0.015), (0.06, 0.09, 0.07), nl2, nq2)
        hs = np.zeros((len(hv), 8), dtype=np.float32)
        hs[:, 0:4] = (2, 0, 0, 0)
        hs[:, 4] = 1.0
        es = np.zeros((len(ev), 8), dtype=np.float32)
        es[:, 0:4] = (1, 0, 0, 0)
        es[:, 4] = 1.0
        mesh = merge_meshes([(hv, hi, hs), (ev, ei, es)])
        pivot = (cx, 1.48, cz)
        phase = float(rng.uniform(0.0, 1.0))
        base = nod_turn_bones(pivot, nod_deg=float(rng.uniform(10, 30)), turn_deg=float(rng.uniform(10, 40)))
        bones = (lambda b, ph: (lambda t: b(t + ph)))(base, phase)
        p = mesh.vertices[:, :3].astype(np.float64)
        lo, hi_ = p.min(0), p.max(0)
        extent = float((hi_ - lo).max()) + 2 * 0.02
        objs.append(SceneObject(asset, st, bones, mesh, bones, (dims,) * 3, extent / dims, (lo + hi_) / 2, follow_bone=2))
    sc = Scene(f"batched_{num_objects}obj", objs, frames=frames)
    return sc
