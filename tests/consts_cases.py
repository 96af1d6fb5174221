"""Seeded cases for the per-frame constant block: TressFXSimulationSettings values (every field that
UpdateSimulationParameters reads, wind off in about a fifth of them), time step, vertices per
strand, follow hairs per guide and simulation frame (the wind varies with the frame)."""
from __future__ import annotations

import numpy as np


def cases(seed: int, count: int) -> list[tuple[dict, float, int, int, int]]:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = rng.normal(size=3)
        if rng.uniform() < 0.1:
            d = np.array([1.0, 0.0, 0.0]) if rng.uniform() < 0.5 else np.array([0.0, 0.0, 0.0])
        st = dict(vsp_coeff=float(rng.uniform(0, 1)), vsp_accel_threshold=float(rng.uniform(0, 3)),
                  local_constraint_stiffness=float(rng.uniform(0, 1)),
                  local_constraints_iterations=int(rng.integers(0, 5)),
                  global_constraint_stiffness=float(rng.uniform(0, 1)),
                  global_constraints_range=float(rng.uniform(0, 1)),
                  length_constraints_iterations=int(rng.integers(0, 5)), damping=float(rng.uniform(0, 0.2)),
                  gravity_magnitude=float(rng.uniform(0, 10)), tip_separation=float(rng.uniform(0, 1)),
                  wind_magnitude=float(rng.uniform(0, 5)) if rng.uniform() < 0.8 else 0.0,
                  wind_direction=tuple(float(x) for x in d))
        n = int(rng.choice([4, 8, 16, 32, 64]))
        F = int(rng.integers(0, 5))
        frame = int(rng.integers(0, 4)) if rng.uniform() < 0.1 else int(rng.integers(0, 20000))
        dt = float(rng.choice([1 / 60, 1 / 30, 0.01]))
        out.append((st, dt, n, F, frame))
    return out
