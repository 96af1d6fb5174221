"""Benchmark: hair vertex-steps/s of TressFX strand simulation + SDF collision on one GB300.

A step is one full frame of the per-frame pipeline on the synthetic "head" workload (20,000 guide
strands x 32 vertices, 4 follow hairs per guide = 3.2 M vertices; 20k-triangle head mesh skinned
by 3 joints; SDF 64^3 rebuilt every frame; 3 local-shape + 3 length iterations, VSP, wind with
+-30 % noise): skin the collision mesh, rebuild the SDF, simulate, collide.

value  = vertices simulated per second over the timed frames, device time (CUDA events recorded on
         the library's own stream), inputs resident in HBM.
e2e    = the same metric through the public API with host buffers: every frame uploads its
         constants (settings + bone matrices) and reads the simulated positions back into pinned
         host memory; host wall clock with a synchronize per frame.
--impl reference times the oracle (the CPU restatement of the reference shaders) on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))


# ------------------------------------------------------------------------------------------ utils
def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self._t:
                self._t.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------------------------ workload
def make_scene(name: str):
    from tressfx_gb300 import synthetic as S
    if name == "head":
        return S.scene_head()
    if name == "fur":
        return S.scene_fur()
    if name == "small":
        return S.scene_small()
    raise SystemExit(f"unknown config {name}")


def algorithmic_bytes(scene) -> dict[str, float]:
    """Algorithmic HBM bytes per frame of each kernel (each buffer element touched once)."""
    out: dict[str, float] = {}
    for o in scene.objects:
        a = o.asset
        G, n, F = a.num_guide_strands, a.verts_per_strand, a.follow_per_guide
        Vg, S, Vt = G * n, G, a.num_vertices
        st = o.settings
        cpu_it = st["local_constraints_iterations"] if n < 64 else 1
        add = lambda k, v: out.__setitem__(k, out.get(k, 0.0) + v)  # noqa: E731
        add("IntegrationAndGlobalShapeConstraints", 96 * Vg + 32 * S)
        add("CalculateStrandLevelData", 196 * S)
        add("VelocityShockPropagation", 64 * Vg * (n - 2) / n + 32 * S)
        add("LocalShapeConstraints", cpu_it * (48 * Vg + 16 * S))
        add("LengthConstriantsWindAndCollision", 68 * Vg)
        add("UpdateFollowHairVertices", (32 * Vg * (1 + F) + 16 * F * S) if F > 0 else 0)
        if o.mesh is not None:
            C_ = int(np.prod(o.sdf_dims))
            T, Vm = o.mesh.num_triangles, len(o.mesh.vertices)
            add("BoneSkinning", 96 * Vm)
            add("InitializeSignedDistanceField", 4 * C_)
            add("ConstructSignedDistanceField", 12 * T + 32 * Vm + 4 * C_)
            add("FinalizeSignedDistanceField", 8 * C_)
            add("CollideHairVerticesWithSdf", 16 * Vt + 4 * C_)
    return out


# ------------------------------------------------------------------------------------------ GPU arm
def run_gpu(args) -> dict:
    from tressfx_gb300 import _capi as A
    from tressfx_gb300.api import Context
    from tressfx_gb300.headless import FrameInputs, PlainPipeline
    from tressfx_gb300.synthetic import margin_world

    device = int(os.environ.get("LOCAL_RANK", "0"))
    scene = make_scene(args.config)
    ctx = Context(device)
    pipe = PlainPipeline(ctx, scene)
    vpf = scene.vertices_per_frame

    total = args.warmup + args.steps
    inputs = [FrameInputs(scene, f) for f in range(total + args.steps)]

    def frame(fin, stamps: bool) -> None:
        pipe.prepare(fin)
        st = ctx.timestamp if stamps else (lambda name: None)
        for m, s, mb, g in zip(pipe.meshes, pipe.sdfs, fin.mesh_bones, fin.grids):
            if m is not None:
                st("BoneSkinning>"); m.skin(mb); st("BoneSkinning<")
                for k, nm in ((A.K_SDF_INITIALIZE, "InitializeSignedDistanceField"),
                              (A.K_SDF_CONSTRUCT, "ConstructSignedDistanceField"),
                              (A.K_SDF_FINALIZE, "FinalizeSignedDistanceField")):
                    st(nm + ">"); s.dispatch(k, g); st(nm + "<")
        for h in pipe.hair:
            h.update_constant_buffer()
        names = ["IntegrationAndGlobalShapeConstraints", "CalculateStrandLevelData", "VelocityShockPropagation",
                 "LocalShapeConstraints", "LengthConstriantsWindAndCollision", "UpdateFollowHairVertices"]
        for k, nm in zip(pipe.sim.STAGES, names):
            st(nm + ">")
            for h in pipe.hair:
                h.dispatch(k, h.cpu_local_iterations if k == A.K_LOCAL_SHAPE_CONSTRAINTS else 1)
            st(nm + "<")
        for h in pipe.hair:
            h.increase_simulation_frame()
        for h, s, o, g in zip(pipe.hair, pipe.sdfs, scene.objects, fin.grids):
            if s is not None:
                st("CollideHairVerticesWithSdf>"); s.collide(h, g, margin_world(o, g)); st("CollideHairVerticesWithSdf<")

    launches_per_frame = 0
    for o in scene.objects:
        it = o.settings["local_constraints_iterations"] if o.asset.verts_per_strand < 64 else 1
        launches_per_frame += 5 + it + (1 if o.asset.follow_per_guide > 0 else 0)
        if o.mesh is not None:
            launches_per_frame += 5

    for f in range(args.warmup):
        frame(inputs[f], False)
    ctx.synchronize()
    ctx.timestamps()

    # ---- device-timed region (stage stamps double as per-kernel timers)
    with ClockSampler(device) as clocks:
        ctx.timestamp("start")
        for f in range(args.warmup, total):
            frame(inputs[f], True)
        ctx.timestamp("end")
        ctx.synchronize()
    stamps = ctx.timestamps(4096)
    t_ms = stamps[-1][1] - stamps[0][1]
    per_kernel: dict[str, list[float]] = {}
    open_t: dict[str, float] = {}
    for name, t in stamps[1:-1]:
        base, edge = name[:-1], name[-1]
        if edge == ">":
            open_t[base] = t
        else:
            per_kernel.setdefault(base, []).append(t - open_t.pop(base))

    # ---- end-to-end through the public API with host buffers
    from tressfx_gb300.api import PinnedArray
    pinned = [PinnedArray((h.num_vertices, 4), np.float32) for h in pipe.hair]
    e2e_frames = args.steps
    d2h = sum(p.array.nbytes for p in pinned)
    h2d = 0
    for h in pipe.hair:
        h2d += 128 + 64 * h.num_bones
    for o in scene.objects:
        if o.mesh is not None:
            h2d += 64 * 3
    ctx.synchronize()
    t0 = time.perf_counter()
    for f in range(total, total + e2e_frames):
        frame(inputs[f], False)
        for h, p in zip(pipe.hair, pinned):
            h.read_async(A.BUF_POSITIONS, p.array)
        ctx.synchronize()
    e2e_s = time.perf_counter() - t0
    for p in pinned:
        p.free()

    value = vpf * args.steps / (t_ms * 1e-3)
    e2e = vpf * e2e_frames / e2e_s
    peaks = load_peaks()
    algo = algorithmic_bytes(scene)
    kern_ms = {k: float(np.mean(v)) for k, v in per_kernel.items()}
    dom = max(kern_ms, key=lambda k: kern_ms[k])
    dom_bytes = algo.get(dom, 0.0)
    achieved = dom_bytes / (kern_ms[dom] * 1e-3) / 1e9 if kern_ms[dom] > 0 else 0.0
    res = {
        "value": value, "ms_per_step": t_ms / args.steps, "e2e_value": e2e, "e2e_ms_per_step": e2e_s * 1e3 / e2e_frames,
        "h2d": h2d, "d2h": d2h, "kernel_ms": kern_ms, "dominant": dom, "dominant_bytes": dom_bytes,
        "achieved_gbs": achieved, "peak_gbs": peaks["hbm_gbs"], "peak_source": peaks["source"],
        "clocks": clocks.summary(), "launches": launches_per_frame * args.steps, "scene": scene, "algo": algo,
    }
    pipe.close()
    ctx.close()
    return res


# ------------------------------------------------------------------------------------------ CPU legs
def oracle_frames(scene, frames: int, min_seconds: float, max_seconds: float, threads: int) -> tuple[float, int]:
    """Runs the oracle pipeline; returns (seconds, frames) of the bounded sample."""
    from oracle.scene_driver import OraclePipeline
    from tressfx_gb300.headless import FrameInputs
    pipe = OraclePipeline(scene, np.float32, threads)
    pipe.step(FrameInputs(scene, 0))   # untimed first frame (reset pose)
    done, t0 = 0, time.perf_counter()
    while True:
        pipe.step(FrameInputs(scene, 1 + done))
        done += 1
        el = time.perf_counter() - t0
        if done >= frames and el >= min_seconds or el >= max_seconds:
            return el, done


def run_reference(args) -> dict:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return {}
    scene = make_scene(args.config)
    threads = os.cpu_count() or 1
    from oracle.scene_driver import OraclePipeline
    from tressfx_gb300.headless import FrameInputs
    pipe = OraclePipeline(scene, np.float32, threads)
    for f in range(args.warmup):
        pipe.step(FrameInputs(scene, f))
    t0 = time.perf_counter()
    for f in range(args.warmup, args.warmup + args.steps):
        pipe.step(FrameInputs(scene, f))
    el = time.perf_counter() - t0
    v = scene.vertices_per_frame * args.steps / el
    return {"value": v, "ms_per_step": el * 1e3 / args.steps, "threads": threads, "scene": scene}


# ------------------------------------------------------------------------------------------ main
def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="head", choices=["head", "fur", "small"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo" if args.impl == "reference" else "nccl")

    metric = "hair vertex-steps/s"
    workload = {"head": "head 20000x32 F=4 (3.2M verts), 20k-tri mesh, SDF 64^3, 3 local + 3 length iters, wind",
                "fur": "fur 200000x16 (3.2M verts), 50k-tri torso, SDF 128^3, 2 local + 2 length iters",
                "small": "plain small 2048x16, no SDF"}[args.config]

    if args.impl == "reference":
        r = run_reference(args)
        if rank == 0:
            line = {"metric": metric, "value": r["value"], "unit": "vertex-steps/s", "n_gpus": args.gpus,
                    "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                    "data": "synthetic (seeded)", "impl": "reference",
                    "config": {"workload": workload, "parallelism": "replicas", "l2": "inputs larger than L2"},
                    "cpu_baseline": {"value": r["value"], "unit": "vertex-steps/s", "cores": r["threads"], "kind": "port",
                                     "sample": f"{args.steps} full frames of the workload after {args.warmup} warm-up frames"},
                    "e2e": {"value": r["value"], "unit": "vertex-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
            print(json.dumps(line), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return

    r = run_gpu(args)
    # max over ranks of the device time
    ms = r["ms_per_step"]
    if dist is not None:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=f"cuda:{int(os.environ.get('LOCAL_RANK', '0'))}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = r["scene"].vertices_per_frame * world / (ms * 1e-3)

    if rank == 0:
        cpu = None
        if world == 1 or rank == 0:
            threads = os.cpu_count() or 1
            el, fr = oracle_frames(r["scene"], 1, args.cpu_seconds, 4 * args.cpu_seconds, threads)
            cpu = {"value": r["scene"].vertices_per_frame * fr / el, "unit": "vertex-steps/s", "cores": threads,
                   "kind": "port", "sample": f"{fr} full frames of the workload after one untimed frame ({el:.1f} s)"}
        dom = r["dominant"]
        line = {
            "metric": metric, "value": value, "unit": "vertex-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": workload, "path": "plain (one launch per object per stage)",
                       "parallelism": "replicas" if world > 1 else "single", "l2": "inputs larger than L2 (state 256 MB)"},
            "e2e": {"value": r["e2e_value"], "unit": "vertex-steps/s", "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"]},
            "gpu_launches": r["launches"],
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": r["achieved_gbs"], "peak": r["peak_gbs"],
                         "unit": "GB/s", "frac": r["achieved_gbs"] / r["peak_gbs"], "traffic": None,
                         "peak_source": r["peak_source"], "algorithmic_bytes": r["dominant_bytes"]},
            "kernel_ms": r["kernel_ms"],
            "cpu_baseline": cpu,
            "clocks": r["clocks"],
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
