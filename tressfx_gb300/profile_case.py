"""Runs a few frames of a workload on one path, for profilers (ncu) and quick checks.

    python -m tressfx_gb300.profile_case --config head --path batched --frames 3

No autotuning, no timing, no oracle: exactly `--frames` frames after `--warmup` frames, so a
profiler sees a short, predictable launch list.
"""
from __future__ import annotations

import argparse

from .api import Context
from .headless import BatchedPipeline, FrameInputs, PlainPipeline
from . import synthetic as S


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="head", choices=["head", "fur", "small", "batched"])
    ap.add_argument("--path", default="batched", choices=["batched", "plain"])
    ap.add_argument("--frames", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=2)
    a = ap.parse_args()
    scene = {"head": S.scene_head, "fur": S.scene_fur, "small": S.scene_small, "batched": S.scene_batched}[a.config]()
    ctx = Context(0)
    pipe = BatchedPipeline(ctx, scene) if a.path == "batched" else PlainPipeline(ctx, scene)
    for f in range(a.warmup + a.frames):
        pipe.step(f)
    ctx.synchronize()
    pipe.close()
    ctx.close()
    print(f"{a.config}/{a.path}: {a.warmup + a.frames} frames done")


if __name__ == "__main__":
    main()
