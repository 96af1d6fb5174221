"""Python handles over the C ABI, shaped like the reference's host classes.

``HairObject`` follows TressFXHairObject (src/TressFX/TressFXHairObject.h:85-191): it keeps the
two host constant blocks ``m_SimCB[frame % 2]``, the simulation frame counter, and forwards
UpdateSimulationParameters / UpdateBoneMatrices / UpdateConstantBuffer / ResetPositions /
IncreaseSimulationFrame.  ``Simulation.simulate`` is TressFXSimulation::Simulate
(src/TressFX/TressFXSimulation.cpp:77-112): stage-major, object-minor dispatch order.
``SDFCollision`` is TressFXSDFCollision (src/TressFX/TressFXSDFCollision.cpp:38-221) and
``CollisionMesh`` the skinned mesh of TressFXBoneSkinning (src/TressFX/TressFXBoneSkinning.cpp).
All device work runs in libtfxgb300.so; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as A
from ._capi import check, ptr


class Context:
    """EI_Device + EI_CommandContext: one CUDA stream on one device."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(A.lib().tfx_context_create(device, C.byref(h)), "tfx_context_create")
        self.handle = h
        self.device = device

    def synchronize(self) -> None:
        check(A.lib().tfx_context_synchronize(self.handle), "tfx_context_synchronize")

    @property
    def stream(self) -> int:
        return A.lib().tfx_context_stream(self.handle) or 0

    def timestamp(self, name: str) -> None:
        check(A.lib().tfx_context_timestamp(self.handle, name.encode()), "tfx_context_timestamp")

    def timestamps(self, max_count: int = 256) -> list[tuple[str, float]]:
        names = (C.c_char * 64 * max_count)()
        ms = (C.c_float * max_count)()
        n = C.c_int()
        check(A.lib().tfx_context_timestamps(self.handle, names, ms, max_count, C.byref(n)), "tfx_context_timestamps")
        return [(bytes(names[i]).split(b"\0")[0].decode(), float(ms[i])) for i in range(n.value)]

    def close(self) -> None:
        if getattr(self, "handle", None):
            A.lib().tfx_context_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class PinnedArray:
    """A numpy array over page-locked host memory from tfx_host_alloc."""

    def __init__(self, shape, dtype=np.float32):
        dt = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dt.itemsize
        p = C.c_void_p()
        check(A.lib().tfx_host_alloc(nbytes, C.byref(p)), "tfx_host_alloc")
        self._ptr = p.value
        buf = (C.c_byte * nbytes).from_address(self._ptr)
        self.array = np.frombuffer(buf, dtype=dt).reshape(shape)

    def free(self) -> None:
        if self._ptr:
            self.array = None
            A.lib().tfx_host_free(self._ptr)
            self._ptr = None


def default_settings() -> A.SimSettings:
    s = A.SimSettings()
    check(A.lib().tfx_sim_settings_default(C.byref(s)), "tfx_sim_settings_default")
    return s


def fill_sim_params(params: A.SimParams, settings: A.SimSettings, dt: float, n: int, F: int, frame: int) -> int:
    """TressFXHairObject::UpdateSimulationParameters on a constant block; returns CPU local iterations."""
    it = C.c_int32()
    check(A.lib().tfx_fill_sim_params(C.byref(params), C.byref(settings), dt, n, F, frame, C.byref(it)),
          "tfx_fill_sim_params")
    return it.value


class SimConstants:
    """Host half of TressFXHairObject: the two constant blocks m_SimCB[frame % 2], the simulation
    frame counter and the CPU local-shape iteration count (TressFXHairObject.cpp:366-437,
    TressFXHairObject.h:104,129).  Needs no device."""

    def __init__(self, n: int, F: int):
        self.n, self.F = n, F
        self.sim_cb = [A.SimParams(), A.SimParams()]
        self.frame = 0
        self.cpu_local_iterations = 0
        self.num_bones = 0
        self.reset_positions()

    def reset_positions(self) -> None:
        self.sim_cb[self.frame % 2].reset_positions = 1.0

    def update_simulation_parameters(self, settings: A.SimSettings, dt: float) -> None:
        self.cpu_local_iterations = fill_sim_params(self.sim_cb[self.frame % 2], settings, dt, self.n, self.F, self.frame)

    def update_bone_matrices(self, mats: np.ndarray) -> None:
        mats = np.ascontiguousarray(mats, dtype=np.float32).reshape(-1, 16)
        k = min(len(mats), A.TFX_MAX_BONES)
        self.sim_cb[self.frame % 2].bones_view()[:k] = mats[:k]
        self.num_bones = max(self.num_bones, k)

    def increase_simulation_frame(self) -> None:
        self.sim_cb[self.frame % 2].reset_positions = 0.0
        self.frame += 1

    def current_params(self) -> A.SimParams:
        return self.sim_cb[self.frame % 2]


class HairObject(SimConstants):
    """TressFXHairObject over a tfx_hair handle."""

    def __init__(self, ctx: Context, asset: "HairAsset"):
        self.ctx = ctx
        self.G, self.n, self.F = asset.num_guide_strands, asset.verts_per_strand, asset.follow_per_guide
        desc = A.HairDesc(self.G, self.n, self.F, 0)
        h = C.c_void_p()
        check(A.lib().tfx_hair_create(ctx.handle, C.byref(desc), ptr(asset.positions), ptr(asset.tangents),
                                      ptr(asset.rest_lengths), ptr(asset.follow_root_offsets),
                                      ptr(asset.bone_skinning), C.byref(h)), "tfx_hair_create")
        self.handle = h
        self.num_vertices = self.G * (self.F + 1) * self.n
        self.num_strands = self.G * (self.F + 1)
        SimConstants.__init__(self, self.n, self.F)

    def update_constant_buffer(self) -> None:
        check(A.lib().tfx_hair_update_constants(self.handle, C.byref(self.sim_cb[self.frame % 2]), self.num_bones),
              "tfx_hair_update_constants")

    # --- dispatch / buffers ----------------------------------------------------------------
    def dispatch(self, kernel: int, repeat: int = 1) -> None:
        check(A.lib().tfx_hair_dispatch(self.handle, kernel, repeat), "tfx_hair_dispatch")

    def simulate_stages(self) -> None:
        check(A.lib().tfx_hair_simulate(self.handle, self.cpu_local_iterations), "tfx_hair_simulate")

    _SHAPES = {A.BUF_POSITIONS: "v4", A.BUF_POSITIONS_PREV: "v4", A.BUF_POSITIONS_PREV_PREV: "v4", A.BUF_TANGENTS: "v4",
               A.BUF_STRAND_LEVEL_DATA: "s12", A.BUF_INITIAL_POSITIONS: "v4", A.BUF_REST_LENGTHS: "v1",
               A.BUF_FOLLOW_ROOT_OFFSETS: "s4", A.BUF_BONE_SKINNING: "s8"}

    def buffer_shape(self, buf: int) -> tuple[int, ...]:
        kind = self._SHAPES[buf]
        if kind == "v4":
            return (self.num_vertices, 4)
        if kind == "v1":
            return (self.num_vertices,)
        return (self.num_strands, int(kind[1:]))

    def count_nonfinite(self) -> tuple[int, int]:
        """Vertices of Pos and of Prev with a NaN or infinite component (report only)."""
        c = (C.c_int64 * 2)()
        check(A.lib().tfx_hair_count_nonfinite(self.handle, c), "tfx_hair_count_nonfinite")
        return int(c[0]), int(c[1])

    def read(self, buf: int, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.buffer_shape(buf), dtype=np.float32)
        check(A.lib().tfx_hair_read(self.handle, buf, ptr(out), out.nbytes), "tfx_hair_read")
        return out

    def write(self, buf: int, data: np.ndarray) -> None:
        data = np.ascontiguousarray(data, dtype=np.float32)
        check(A.lib().tfx_hair_write(self.handle, buf, ptr(data), data.nbytes), "tfx_hair_write")

    def read_async(self, buf: int, out: np.ndarray) -> None:
        check(A.lib().tfx_hair_read_async(self.handle, buf, ptr(out), out.nbytes), "tfx_hair_read_async")

    def device_buffer(self, buf: int) -> tuple[int, int]:
        p = C.c_void_p()
        n = C.c_size_t()
        check(A.lib().tfx_hair_get_buffer(self.handle, buf, C.byref(p), C.byref(n)), "tfx_hair_get_buffer")
        return p.value, n.value

    def snapshot(self) -> dict[int, np.ndarray]:
        return {b: self.read(b) for b in (A.BUF_POSITIONS, A.BUF_POSITIONS_PREV, A.BUF_POSITIONS_PREV_PREV,
                                          A.BUF_TANGENTS, A.BUF_STRAND_LEVEL_DATA)}

    def restore(self, snap: dict[int, np.ndarray]) -> None:
        for b, a in snap.items():
            self.write(b, a)

    def close(self) -> None:
        if getattr(self, "handle", None):
            A.lib().tfx_hair_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class Simulation:
    """TressFXSimulation: Simulate(objects) in the reference's stage-major order."""

    STAGES = (A.K_INTEGRATION_AND_GLOBAL_SHAPE, A.K_STRAND_LEVEL_DATA, A.K_VELOCITY_SHOCK_PROPAGATION,
              A.K_LOCAL_SHAPE_CONSTRAINTS, A.K_LENGTH_WIND_COLLISION, A.K_UPDATE_FOLLOW_HAIR)

    def simulate(self, objects: list[HairObject]) -> None:
        for o in objects:
            o.update_constant_buffer()
        for k in self.STAGES:
            for o in objects:
                o.dispatch(k, o.cpu_local_iterations if k == A.K_LOCAL_SHAPE_CONSTRAINTS else 1)
        for o in objects:
            o.increase_simulation_frame()


class CollisionMesh:
    """Skinned collision mesh (TressFXBoneSkinning) feeding an SDF."""

    def __init__(self, ctx: Context, vertices: np.ndarray, indices: np.ndarray, skinning: np.ndarray):
        self.ctx = ctx
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 8)
        self.indices = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1)
        self.skinning = np.ascontiguousarray(skinning, dtype=np.float32).reshape(-1, 8)
        h = C.c_void_p()
        check(A.lib().tfx_mesh_create(ctx.handle, ptr(self.vertices), len(self.vertices), ptr(self.indices),
                                      len(self.indices) // 3, ptr(self.skinning), C.byref(h)), "tfx_mesh_create")
        self.handle = h
        sk, ix = C.c_void_p(), C.c_void_p()
        nv, nt = C.c_int32(), C.c_int32()
        check(A.lib().tfx_mesh_get_buffers(h, C.byref(sk), C.byref(ix), C.byref(nv), C.byref(nt)), "tfx_mesh_get_buffers")
        self.skinned_ptr, self.index_ptr, self.num_vertices, self.num_triangles = sk.value, ix.value, nv.value, nt.value

    def skin(self, bone_matrices: np.ndarray) -> None:
        m = np.ascontiguousarray(bone_matrices, dtype=np.float32).reshape(-1, 16)
        check(A.lib().tfx_mesh_skin(self.handle, ptr(m), len(m)), "tfx_mesh_skin")

    def read_skinned(self) -> np.ndarray:
        out = np.empty((self.num_vertices, 8), dtype=np.float32)
        check(A.lib().tfx_mesh_read_skinned(self.handle, ptr(out), out.nbytes), "tfx_mesh_read_skinned")
        return out

    def close(self) -> None:
        if getattr(self, "handle", None):
            A.lib().tfx_mesh_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


def grid_from_bbox(bmin, bmax, num_cells_in_x: int) -> tuple[A.SdfGrid, float, int]:
    g = A.SdfGrid()
    pad = C.c_float()
    alloc = C.c_int64()
    bmin = (C.c_float * 3)(*bmin)
    bmax = (C.c_float * 3)(*bmax)
    check(A.lib().tfx_sdf_grid_from_bbox(bmin, bmax, num_cells_in_x, C.byref(g), C.byref(pad), C.byref(alloc)),
          "tfx_sdf_grid_from_bbox")
    return g, pad.value, alloc.value


class SDFCollision:
    """TressFXSDFCollision: a signed distance grid rebuilt from a bound mesh, collided with hair."""

    def __init__(self, ctx: Context, alloc_cells: int):
        self.ctx = ctx
        h = C.c_void_p()
        check(A.lib().tfx_sdf_create(ctx.handle, int(alloc_cells), C.byref(h)), "tfx_sdf_create")
        self.handle = h
        self.alloc_cells = int(alloc_cells)

    def set_mesh_device(self, vertices_ptr: int, num_vertices: int, indices_ptr: int, num_triangles: int) -> None:
        check(A.lib().tfx_sdf_set_mesh(self.handle, vertices_ptr, num_vertices, indices_ptr, num_triangles),
              "tfx_sdf_set_mesh")

    def bind_mesh(self, mesh: CollisionMesh) -> None:
        self.set_mesh_device(mesh.skinned_ptr, mesh.num_vertices, mesh.index_ptr, mesh.num_triangles)

    def update(self, grid: A.SdfGrid) -> None:
        check(A.lib().tfx_sdf_update(self.handle, C.byref(grid)), "tfx_sdf_update")

    def dispatch(self, kernel: int, grid: A.SdfGrid) -> None:
        check(A.lib().tfx_sdf_dispatch(self.handle, kernel, C.byref(grid)), "tfx_sdf_dispatch")

    def collide(self, hair: HairObject, grid: A.SdfGrid, margin_world: float) -> None:
        check(A.lib().tfx_sdf_collide(self.handle, hair.handle, C.byref(grid), float(margin_world)), "tfx_sdf_collide")

    def collide_mixed(self, hair: HairObject, grid: A.SdfGrid, margin_world: float) -> None:
        """CollideHairVerticesWithSdf, the mixed forward / backward difference variant."""
        check(A.lib().tfx_sdf_collide_mixed(self.handle, hair.handle, C.byref(grid), float(margin_world)),
              "tfx_sdf_collide_mixed")

    def read(self, cells: int) -> np.ndarray:
        out = np.empty(cells, dtype=np.uint32)
        check(A.lib().tfx_sdf_read(self.handle, ptr(out), out.nbytes), "tfx_sdf_read")
        return out

    def write(self, data: np.ndarray) -> None:
        data = np.ascontiguousarray(data, dtype=np.uint32)
        check(A.lib().tfx_sdf_write(self.handle, ptr(data), data.nbytes), "tfx_sdf_write")

    def close(self) -> None:
        if getattr(self, "handle", None):
            A.lib().tfx_sdf_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


def mc_default_tables() -> tuple[np.ndarray, np.ndarray]:
    """The library's marching-cubes tables: edge[256] and triangles[256, 16] (-1 terminated)."""
    e = np.zeros(256, np.int32)
    t = np.zeros((256, 16), np.int32)
    check(A.lib().tfx_mc_default_tables(ptr(e), ptr(t)), "tfx_mc_default_tables")
    return e, t


class SDFMarchingCubes:
    """TressFXSDFMarchingCubes: the iso-surface of a signed distance grid as a device triangle soup of
    {float4 position, float4 normal} vertices, in cell-index order."""

    def __init__(self, ctx: Context, max_vertices: int = 128 * 1024, max_cells: int = 1 << 21):
        self.ctx = ctx
        h = C.c_void_p()
        check(A.lib().tfx_mc_create(ctx.handle, int(max_vertices), int(max_cells), C.byref(h)), "tfx_mc_create")
        self.handle = h
        self.max_vertices = int(max_vertices)

    def set_tables(self, edge_table=None, tri_table=None) -> None:
        if edge_table is None:
            check(A.lib().tfx_mc_set_tables(self.handle, None, None), "tfx_mc_set_tables")
            return
        e = np.ascontiguousarray(edge_table, dtype=np.int32).reshape(256)
        t = np.ascontiguousarray(tri_table, dtype=np.int32).reshape(256 * 16)
        check(A.lib().tfx_mc_set_tables(self.handle, ptr(e), ptr(t)), "tfx_mc_set_tables")

    def set_iso_level(self, iso_level_cells: float) -> None:
        check(A.lib().tfx_mc_set_iso_level(self.handle, float(iso_level_cells)), "tfx_mc_set_iso_level")

    def update(self, sdf: SDFCollision, grid: A.SdfGrid) -> None:
        check(A.lib().tfx_mc_update(self.handle, sdf.handle, C.byref(grid)), "tfx_mc_update")

    def run(self, sdf_device_ptr: int, grid: A.SdfGrid) -> None:
        check(A.lib().tfx_mc_run(self.handle, sdf_device_ptr, C.byref(grid)), "tfx_mc_run")

    def buffers(self) -> tuple[int, int]:
        v, n = C.c_void_p(), C.c_void_p()
        check(A.lib().tfx_mc_get_buffers(self.handle, C.byref(v), C.byref(n)), "tfx_mc_get_buffers")
        return v.value, n.value

    def read(self, vertices: int | None = None) -> tuple[np.ndarray, int]:
        """(vertices[:vertices] as (N, 8) float32, the counter)."""
        nv = self.max_vertices if vertices is None else int(vertices)
        out = np.empty((nv, 8), np.float32)
        cnt = C.c_int32()
        check(A.lib().tfx_mc_read(self.handle, ptr(out), out.nbytes, C.byref(cnt)), "tfx_mc_read")
        return out, cnt.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            A.lib().tfx_mc_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """tfx_batch: many hair objects and their SDFs advanced by one CUDA-graph launch per frame."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        check(A.lib().tfx_batch_create(ctx.handle, C.byref(h)), "tfx_batch_create")
        self.handle = h
        self._keep = []

    def add_sdf(self, sdf: SDFCollision, mesh: CollisionMesh | None, dims) -> int:
        i = C.c_int()
        check(A.lib().tfx_batch_add_sdf(self.handle, sdf.handle, mesh.handle if mesh is not None else None,
                                        int(dims[0]), int(dims[1]), int(dims[2]), C.byref(i)), "tfx_batch_add_sdf")
        self._keep += [sdf, mesh]
        return i.value

    def add_hair(self, hair: HairObject, sdf_index: int = -1) -> int:
        i = C.c_int()
        check(A.lib().tfx_batch_add_hair(self.handle, hair.handle, sdf_index, C.byref(i)), "tfx_batch_add_hair")
        self._keep.append(hair)
        return i.value

    def add_hair_collision(self, hair_index: int, sdf_index: int) -> None:
        """Hair object `hair_index` also collides with SDF `sdf_index`, after its earlier SDFs."""
        check(A.lib().tfx_batch_add_hair_collision(self.handle, int(hair_index), int(sdf_index)),
              "tfx_batch_add_hair_collision")

    def build(self) -> None:
        check(A.lib().tfx_batch_build(self.handle, 0), "tfx_batch_build")

    EXPANDED_GRIDS, OVERLAP_SDF, SDF_BLOCK, SPLIT_SWEEPS, FOLLOW_FORM, WAIT_POLLS, SDF_FORM = 1, 2, 3, 4, 5, 6, 7

    def set_option(self, option: int, value: int) -> None:
        check(A.lib().tfx_batch_set_option(self.handle, option, value), "tfx_batch_set_option")

    def get_option(self, option: int) -> int:
        v = C.c_int()
        check(A.lib().tfx_batch_get_option(self.handle, option, C.byref(v)), "tfx_batch_get_option")
        return v.value

    def autotune(self, frames: int = 3) -> None:
        check(A.lib().tfx_batch_autotune(self.handle, frames), "tfx_batch_autotune")

    def set_hair_constants(self, index: int, params: A.SimParams, num_bones: int, cpu_local_iterations: int) -> None:
        check(A.lib().tfx_batch_set_hair_constants(self.handle, index, C.byref(params), num_bones, cpu_local_iterations),
              "tfx_batch_set_hair_constants")

    def set_sdf_frame(self, index: int, grid: A.SdfGrid, margin_world: float) -> None:
        check(A.lib().tfx_batch_set_sdf_frame(self.handle, index, C.byref(grid), float(margin_world)),
              "tfx_batch_set_sdf_frame")

    def set_mesh_bones(self, index: int, bones: np.ndarray) -> None:
        b = np.ascontiguousarray(bones, dtype=np.float32).reshape(-1, 16)
        check(A.lib().tfx_batch_set_mesh_bones(self.handle, index, ptr(b), len(b)), "tfx_batch_set_mesh_bones")

    def run(self) -> None:
        check(A.lib().tfx_batch_run(self.handle), "tfx_batch_run")

    def synchronize(self) -> None:
        """Waits for the queued frames; raises TfxError(TFX_ERR_TIMEOUT) once if one of them timed out."""
        check(A.lib().tfx_batch_synchronize(self.handle), "tfx_batch_synchronize")

    READBACK_XYZW, READBACK_XYZ = 0, 1

    def readback(self, host_ptrs: list[int], fmt: int = 0) -> int:
        """Queues the copy of every hair object's positions into host memory (float4, or packed xyz with
        fmt = READBACK_XYZ); returns a ticket."""
        arr = (C.c_void_p * len(host_ptrs))(*host_ptrs)
        tk = C.c_int64()
        check(A.lib().tfx_batch_readback(self.handle, arr, len(host_ptrs), int(fmt), C.byref(tk)), "tfx_batch_readback")
        return tk.value

    def wait_readback(self, ticket: int) -> None:
        check(A.lib().tfx_batch_wait_readback(self.handle, int(ticket)), "tfx_batch_wait_readback")

    def profile_frame(self) -> list[float]:
        ms = (C.c_float * 16)()
        n = C.c_int()
        check(A.lib().tfx_batch_profile_frame(self.handle, ms, 16, C.byref(n)), "tfx_batch_profile_frame")
        return [float(ms[i]) for i in range(min(n.value, 16))]

    def describe(self) -> tuple[str, int]:
        buf = C.create_string_buffer(1024)
        n = C.c_int32()
        check(A.lib().tfx_batch_describe(self.handle, buf, 1024, C.byref(n)), "tfx_batch_describe")
        return buf.value.decode(), n.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            A.lib().tfx_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class NeuralSDF:
    """tfx_nsdf: the learned collision proxy (pose-conditioned neural SDF) over the C ABI."""

    def __init__(self, ctx: Context, box_min, box_max, cell_size: float, band_cells: float = 3.0,
                 pose_scale: float = 1.0 / 0.7, sphere=None, seed: int = 1, max_samples: int = 1 << 20,
                 max_eval_samples: int = 1 << 18, contact_slack_cells: float = 1.0):
        self.ctx = ctx
        d = A.NsdfDesc()
        for k in range(3):
            d.box_min[k], d.box_max[k] = float(box_min[k]), float(box_max[k])
        d.cell_size, d.band_cells, d.pose_scale = float(cell_size), float(band_cells), float(pose_scale)
        if sphere is not None:
            d.sphere_center[0], d.sphere_center[1], d.sphere_center[2] = (float(x) for x in sphere[:3])
            d.sphere_radius = float(sphere[3])
        d.seed, d.max_samples, d.max_eval_samples = int(seed), int(max_samples), int(max_eval_samples)
        d.contact_slack_cells = float(contact_slack_cells)
        h = C.c_void_p()
        check(A.lib().tfx_nsdf_create(ctx.handle, C.byref(d), C.byref(h)), "tfx_nsdf_create")
        self.handle = h
        self.cell_size = float(cell_size)

    def add_samples(self, pool: int, mesh: CollisionMesh, sdf: SDFCollision, grid: A.SdfGrid, bones: np.ndarray,
                    pose, count: int, sphere=None, sigma_cells: float = 1.5) -> None:
        b = np.ascontiguousarray(bones, dtype=np.float32).reshape(-1, 16)
        p = (C.c_float * 3)(*[float(x) for x in pose])
        sp = (C.c_float * 4)(*[float(x) for x in sphere]) if sphere is not None else None
        check(A.lib().tfx_nsdf_add_samples(self.handle, pool, mesh.handle, sdf.handle, C.byref(grid), ptr(b), len(b), p,
                                           sp, int(count), float(sigma_cells)), "tfx_nsdf_add_samples")

    def train(self, steps: int, batch: int = 8192, lr: float = 1e-3) -> float:
        loss = C.c_float()
        check(A.lib().tfx_nsdf_train(self.handle, int(steps), int(batch), float(lr), C.byref(loss)), "tfx_nsdf_train")
        return float(loss.value)

    def evaluate(self, pool: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        _, tr, ev, _ = self.info()
        n = tr if pool == 0 else ev
        pred, tgt, w = (np.empty(n, np.float32) for _ in range(3))
        cnt = C.c_int64()
        check(A.lib().tfx_nsdf_evaluate(self.handle, pool, ptr(pred), ptr(tgt), ptr(w), n, C.byref(cnt)),
              "tfx_nsdf_evaluate")
        return pred[:cnt.value], tgt[:cnt.value], w[:cnt.value]

    def set_inference(self, form: int) -> None:
        """1: the forward pass on tcgen05 (default); 0: on mma.sync."""
        check(A.lib().tfx_nsdf_set_inference(self.handle, int(form)), "tfx_nsdf_set_inference")

    def query_device(self, points_ptr: int, count: int, pose, out_ptr: int) -> None:
        p = (C.c_float * 3)(*[float(x) for x in pose])
        check(A.lib().tfx_nsdf_query(self.handle, points_ptr, int(count), p, out_ptr), "tfx_nsdf_query")

    def collide(self, hair: HairObject, sdf: SDFCollision, grid: A.SdfGrid, margin_world: float, pose,
                band: bool = False) -> int | None:
        p = (C.c_float * 3)(*[float(x) for x in pose])
        n = C.c_int32()
        check(A.lib().tfx_nsdf_collide(self.handle, hair.handle, sdf.handle, C.byref(grid), float(margin_world), p,
                                       C.byref(n) if band else None), "tfx_nsdf_collide")
        return n.value if band else None

    def set_samples(self, pool: int, samples: np.ndarray) -> None:
        """Replaces a pool with (count, 8) float32 records: x, y, z, target cells, 3 pose angles, weight."""
        s = np.ascontiguousarray(samples, dtype=np.float32).reshape(-1, 8)
        check(A.lib().tfx_nsdf_set_samples(self.handle, int(pool), ptr(s), len(s)), "tfx_nsdf_set_samples")

    def gradients(self) -> np.ndarray:
        n = self.info()[0]
        out = np.empty(n, np.float32)
        check(A.lib().tfx_nsdf_get_gradients(self.handle, ptr(out), n), "tfx_nsdf_get_gradients")
        return out

    def params(self) -> np.ndarray:
        n = self.info()[0]
        out = np.empty(n, np.float32)
        check(A.lib().tfx_nsdf_get_params(self.handle, ptr(out), n), "tfx_nsdf_get_params")
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(A.lib().tfx_nsdf_set_params(self.handle, ptr(p), len(p)), "tfx_nsdf_set_params")

    def info(self) -> tuple[int, int, int, int]:
        a, b, c, d = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int32()
        check(A.lib().tfx_nsdf_get_info(self.handle, C.byref(a), C.byref(b), C.byref(c), C.byref(d)), "tfx_nsdf_get_info")
        return a.value, b.value, c.value, d.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            A.lib().tfx_nsdf_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
