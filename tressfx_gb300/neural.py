"""Training and evaluation driver of the learned collision proxy (tfx_nsdf) for a skinned collision
mesh driven by a 3-joint pose: training data from grid SDFs that the library builds at sampled poses,
then the network's distance error against held-out poses' grids, in cells."""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .api import CollisionMesh, Context, NeuralSDF, SDFCollision
from . import synthetic as S


@dataclass
class ProxyReport:
    train_poses: int
    samples: int
    steps: int
    final_loss: float
    train_seconds: float
    error_mean_cells: float
    error_p99_cells: float
    error_max_cells: float
    eval_points: int


def pose_grid(obj: S.SceneObject, bones: np.ndarray):
    return S.sdf_grid_for(obj, bones)


def normalisation(obj: S.SceneObject, pivot=S.NECK_PIVOT, angle_max: float = math.radians(40.0)):
    """A cube around the pivot holding the grid at every pose of the range, and the mesh's sphere."""
    half = 0.5 * obj.sdf_dims[0] * obj.sdf_cell
    reach = float(np.linalg.norm(np.asarray(obj.sdf_center0) - np.asarray(pivot))) + half
    lo = np.asarray(pivot) - reach
    hi = np.asarray(pivot) + reach
    p = obj.mesh.vertices[:, :3].astype(np.float64)
    c = p.mean(0)
    r = float(np.linalg.norm(p - c, axis=1).max())
    return lo, hi, c, r


def posed_sphere(centre_rest, radius, bones: np.ndarray, bone: int = 2):
    M = bones[bone].reshape(4, 4).astype(np.float64)
    c = np.concatenate([np.asarray(centre_rest, np.float64), [1.0]]) @ M
    return [c[0], c[1], c[2], radius * 1.1]


def train_proxy(ctx: Context, obj: S.SceneObject, poses: int = 512, samples_per_pose: int = 8192,
                eval_poses: int = 32, eval_samples_per_pose: int = 8192, steps: int = 3000, batch: int = 8192,
                lr: float = 2e-3, band_cells: float = 3.0, seed: int = 5,
                angle_max: float = math.radians(40.0), contact_slack_cells: float = 1.0) -> tuple[NeuralSDF, ProxyReport]:
    import time
    rng = np.random.default_rng(seed)
    lo, hi, c, r = normalisation(obj)
    nsdf = NeuralSDF(ctx, lo, hi, obj.sdf_cell, band_cells=band_cells, pose_scale=1.0 / angle_max, seed=seed,
                     max_samples=poses * samples_per_pose, max_eval_samples=max(eval_poses * eval_samples_per_pose, 1),
                     contact_slack_cells=contact_slack_cells)
    m = obj.mesh
    mesh = CollisionMesh(ctx, m.vertices, m.indices, m.skinning)
    sdf = SDFCollision(ctx, int(np.prod(obj.sdf_dims)))
    for pool, count, per in ((0, poses, samples_per_pose), (1, eval_poses, eval_samples_per_pose)):
        for _ in range(count):
            ang = rng.uniform(-angle_max, angle_max, 3)
            bones = S.pose_bones(S.NECK_PIVOT, ang)
            g = pose_grid(obj, bones)
            nsdf.add_samples(pool, mesh, sdf, g, bones, ang, per, sphere=posed_sphere(c, r, bones))
    ctx.synchronize()
    t0 = time.perf_counter()
    loss = nsdf.train(steps, batch, lr)
    ctx.synchronize()
    dt = time.perf_counter() - t0
    pred, tgt, w = nsdf.evaluate(1)
    sel = (w > 0) & (np.abs(tgt) < band_cells - 0.5)
    err = np.abs(pred[sel] - tgt[sel])
    rep = ProxyReport(poses, poses * samples_per_pose, steps, loss, dt, float(err.mean()) if err.size else float("nan"),
                      float(np.percentile(err, 99)) if err.size else float("nan"),
                      float(err.max()) if err.size else float("nan"), int(sel.sum()))
    mesh.close()
    sdf.close()
    return nsdf, rep
