"""Replays a golden fixture (tests/golden/*.npz) on one backend and checks every recorded output.

A fixture holds the inputs of a short run (asset arrays, per-frame constant blocks, collision mesh,
per-frame mesh bones, SDF grids and margins) and SHA-256 digests of the state after each recorded
kernel, written by tests/golden/make_golden.py from the reference's own shaders compiled as C++.
Backends: the oracle (CPU) and the CUDA library (GPU).
"""
from __future__ import annotations

import ctypes as C
import hashlib
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
STATE_KEYS = ("pos", "prev", "prevprev", "tan", "sld")


def digest(*arrays: np.ndarray) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype=np.float32).tobytes() if a.dtype != np.uint32 else
                 np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def state_digest(st: dict) -> str:
    return digest(*[st[k] for k in STATE_KEYS])


# arrays a fixture may take from another fixture (key "inputs_from") instead of holding them itself
INPUT_KEYS = ("positions", "tangents", "rest_lengths", "follow_root_offsets", "bone_skinning", "mesh_vertices",
              "mesh_indices", "mesh_skinning")


def load(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz", allow_pickle=False) as z:
        fx = {k: z[k] for k in z.files}
    if "inputs_from" in fx:
        with np.load(GOLDEN / f"{fx['inputs_from']}.npz", allow_pickle=False) as z:
            for k in INPUT_KEYS:
                fx[k] = z[k]
        n = int(fx["counts"][1])
        fx["positions"] = fx["positions"].reshape(-1, 4)
        fx["tangents"] = fx["tangents"].reshape(-1, 4)
        fx["follow_root_offsets"] = fx["follow_root_offsets"].reshape(-1, 4)
        fx["bone_skinning"] = fx["bone_skinning"].reshape(-1, 8)
        assert fx["positions"].shape[0] % n == 0
    return fx


def fixtures() -> list[str]:
    """The frame-sequence fixtures (mc_*.npz hold marching-cubes cases, sim_params_*.npz constant blocks and
    ratboy_*.npz a slice of the shipped asset, each read by its own tests)."""
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith(("mc_", "sim_params_", "ratboy_")))


def sim_params(fx: dict, frame: int):
    from tressfx_gb300 import _capi as A
    p = A.SimParams()
    hdr = fx[f"cb_header_{frame}"]
    C.memmove(C.addressof(p), hdr.ctypes.data, 160)
    b = fx[f"cb_bones_{frame}"]
    p.bones_view()[:len(b)] = b
    return p, len(b)


class Asset:
    def __init__(self, fx: dict):
        self.num_guide_strands, self.verts_per_strand, self.follow_per_guide = (int(x) for x in fx["counts"])
        self.positions = fx["positions"]
        self.tangents = fx["tangents"]
        self.rest_lengths = fx["rest_lengths"]
        self.follow_root_offsets = fx["follow_root_offsets"]
        self.bone_skinning = fx["bone_skinning"]


def grid(fx: dict, frame: int):
    from tressfx_gb300 import _capi as A
    g = A.SdfGrid()
    o = fx[f"grid_origin_{frame}"]
    for i in range(4):
        g.origin[i] = float(o[i])
    g.cell_size = float(fx[f"grid_cell_{frame}"])
    g.num_cells_x, g.num_cells_y, g.num_cells_z = (int(x) for x in fx["grid_dims"])
    return g


def replay(fx: dict, backend) -> list[str]:
    """Runs the fixture on `backend`; returns the list of mismatching checkpoints (empty = pass)."""
    bad = []
    backend.load(Asset(fx), fx)
    frames = int(fx["frames"])
    for f in range(frames):
        p, nb = sim_params(fx, f)
        backend.set_constants(p, nb)
        has_mesh = "mesh_vertices" in fx
        if has_mesh:
            skinned = backend.mesh_skin(fx[f"mesh_bones_{f}"])
            if digest(skinned) != str(fx[f"h_skinned_{f}"]):
                bad.append(f"frame {f} BoneSkinning")
            words = backend.sdf_build(grid(fx, f))
            if digest(words) != str(fx[f"h_sdf_{f}"]):
                bad.append(f"frame {f} SDF")
        for k in (1, 2, 3, 4, 5, 6):
            reps = int(fx[f"cpu_iters_{f}"]) if k == 4 else 1
            for _ in range(reps):
                backend.stage(k)
            key = f"h_stage{k}_{f}"
            if key in fx and state_digest(backend.state()) != str(fx[key]):
                bad.append(f"frame {f} kernel {k}")
        if has_mesh:
            backend.collide(grid(fx, f), float(fx[f"margin_{f}"]))
        if state_digest(backend.state()) != str(fx[f"h_end_{f}"]):
            bad.append(f"frame {f} end")
    return bad


class OracleBackend:
    def load(self, asset, fx):
        import oracle
        self.o = oracle
        self.h = oracle.OracleHair(asset)
        self.fx = fx

    def set_constants(self, p, nb):
        self.p = p

    def stage(self, k):
        self.h.stage(k, self.p)

    def state(self):
        return {k: getattr(self.h, k) for k in STATE_KEYS}

    def mesh_skin(self, bones):
        self.skinned = self.o.mesh_skin(self.fx["mesh_vertices"], self.fx["mesh_skinning"], bones)
        return self.skinned

    def sdf_build(self, g):
        self.words = self.o.sdf_build(g, self.skinned, self.fx["mesh_indices"])
        return self.words

    def collide(self, g, margin):
        self.o.sdf_collide(g, self.words, margin, self.h)


class GpuBackend:
    def __init__(self, ctx):
        self.ctx = ctx

    def load(self, asset, fx):
        from tressfx_gb300.api import CollisionMesh, HairObject, SDFCollision
        self.h = HairObject(self.ctx, asset)
        self.fx = fx
        if "mesh_vertices" in fx:
            self.mesh = CollisionMesh(self.ctx, fx["mesh_vertices"], fx["mesh_indices"], fx["mesh_skinning"])
            self.sdf = SDFCollision(self.ctx, int(np.prod(fx["grid_dims"])))
            self.sdf.bind_mesh(self.mesh)

    def set_constants(self, p, nb):
        self.h.sim_cb[self.h.frame % 2] = p
        self.h.num_bones = nb
        self.h.update_constant_buffer()
        self.h.frame += 1

    def stage(self, k):
        self.h.dispatch(k, 1)

    def state(self):
        from tressfx_gb300 import _capi as A
        return {"pos": self.h.read(A.BUF_POSITIONS), "prev": self.h.read(A.BUF_POSITIONS_PREV),
                "prevprev": self.h.read(A.BUF_POSITIONS_PREV_PREV), "tan": self.h.read(A.BUF_TANGENTS),
                "sld": self.h.read(A.BUF_STRAND_LEVEL_DATA)}

    def mesh_skin(self, bones):
        self.mesh.skin(bones)
        return self.mesh.read_skinned()

    def sdf_build(self, g):
        self.sdf.update(g)
        return self.sdf.read(g.num_cells)

    def collide(self, g, margin):
        self.sdf.collide(self.h, g, margin)

    def close(self):
        for x in ("h", "mesh", "sdf"):
            o = getattr(self, x, None)
            if o is not None:
                o.close()
