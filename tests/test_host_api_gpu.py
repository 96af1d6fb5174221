"""The C++ host classes (include/tressfx/*.h, libtressfx_host.so) driven the way the reference's
sample drives TressFXSimulation / TressFXHairObject / TressFXSDFCollision / TressFXBoneSkinning,
against the Python mirror of the same classes over the same C ABI: every buffer bit-identical after
several animated frames with follow hairs, wind and SDF collision.  The assets come from .tfx /
.tfxbone / .tfxmesh files read by the C++ loaders."""
import ctypes as C
import os
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from asset_files import strands, write_tfx, write_tfxbone, write_tfxmesh

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def read_named(path: Path) -> dict[str, bytes]:
    raw = path.read_bytes()
    out, pos = {}, 0
    while pos < len(raw):
        (nl,) = struct.unpack_from("<I", raw, pos); pos += 4
        name = raw[pos:pos + nl].decode(); pos += nl
        (nb,) = struct.unpack_from("<Q", raw, pos); pos += 8
        out[name] = raw[pos:pos + nb]; pos += nb
    return out


@pytest.fixture(scope="module")
def host_sim(built_lib, tmp_path_factory):
    d = tmp_path_factory.mktemp("host_sim")
    exe = d / "host_sim"
    pkg = ROOT / "tressfx_gb300"
    subprocess.run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "host_sim.cpp"), "-o", str(exe), f"-L{pkg}", "-ltressfx_host",
                    "-ltfxgb300", f"-Wl,-rpath,{pkg}"], check=True, capture_output=True)
    return exe


def mesh_arrays():
    from tressfx_gb300.synthetic import ellipsoid_mesh
    v, idx = ellipsoid_mesh((0.0, 0.0, 0.0), (0.09, 0.1, 0.09), 24, 32)
    v = np.asarray(v, np.float32).reshape(-1, 8)
    rng = np.random.default_rng(5)
    sk = np.zeros((len(v), 8), np.float32)
    sk[:, 0] = 0
    sk[:, 1] = (v[:, 1] > 0).astype(np.float32)          # upper half also follows bone 1
    sk[:, 2] = 2
    sk[:, 4] = 0.6
    sk[:, 5] = np.where(v[:, 1] > 0, 0.4, 0.0)
    sk[:, 6] = rng.random(len(v)).astype(np.float32) * 0.2
    return v, np.asarray(idx, np.uint32).reshape(-1), sk


def test_cpp_host_classes_match_python_mirror(ctx, host_sim, tmp_path):
    from tressfx_gb300 import _capi as A
    from tressfx_gb300.api import CollisionMesh, HairObject, SDFCollision, Simulation, default_settings

    num, n, F, frames = 150, 16, 3, 6
    s = strands(num, n, 11)
    s[:, :, :3] += np.array([0.0, 0.02, 0.0], np.float32)
    write_tfx(tmp_path / "h.tfx", s)
    write_tfxbone(tmp_path / "h.tfxbone", num, 3, 12)
    mv, mi, msk = mesh_arrays()
    write_tfxmesh(tmp_path / "m.tfxmesh", mv, mi, msk, 3)
    out = tmp_path / "out.bin"
    r = subprocess.run([str(host_sim), str(tmp_path / "h.tfx"), str(tmp_path / "h.tfxbone"), str(tmp_path / "m.tfxmesh"),
                        str(F), str(frames), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    d = read_named(out)
    G, n_, F_ = np.frombuffer(d["counts"], np.int32)
    assert (n_, F_) == (n, F) and G == 192

    class Asset:
        pass
    a = Asset()
    a.num_guide_strands, a.verts_per_strand, a.follow_per_guide = int(G), n, F
    a.positions = np.frombuffer(d["positions"], np.float32).copy()
    a.tangents = np.frombuffer(d["tangents"], np.float32).copy()
    a.rest_lengths = np.frombuffer(d["rest_lengths"], np.float32).copy()
    a.follow_root_offsets = np.frombuffer(d["follow_root_offsets"], np.float32).copy()
    a.bone_skinning = np.frombuffer(d["bone_skinning"], np.float32).copy()
    hair = HairObject(ctx, a)
    mesh = CollisionMesh(ctx, mv, mi, msk)
    alloc = int(np.frombuffer(d["sdf_alloc"], np.int32)[3])
    sdf = SDFCollision(ctx, alloc)
    sdf.bind_mesh(mesh)
    st = default_settings()
    st.gravity_magnitude, st.damping = 9.8, 0.035
    st.global_constraint_stiffness, st.global_constraints_range = 0.2, 0.3
    st.local_constraint_stiffness, st.local_constraints_iterations, st.length_constraints_iterations = 0.8, 3, 3
    st.tip_separation, st.wind_magnitude = 0.5, 2.0
    bones = np.frombuffer(d["bones"], np.float32).reshape(frames, 3, 16)
    grids = np.frombuffer(d["grids"], np.float32).reshape(frames, 8)
    ls = np.frombuffer(d["ls_iters"], np.float32)
    sim = Simulation()
    for f in range(frames):
        hair.update_bone_matrices(bones[f])
        hair.update_simulation_parameters(st, np.float32(1.0) / np.float32(60.0))
        assert hair.cpu_local_iterations == int(ls[f])
        mesh.skin(bones[f])
        g = A.SdfGrid()
        g.origin[0], g.origin[1], g.origin[2], g.origin[3] = float(grids[f, 0]), float(grids[f, 1]), float(grids[f, 2]), 0.0
        g.cell_size = float(grids[f, 3])
        g.num_cells_x, g.num_cells_y, g.num_cells_z = int(grids[f, 4]), int(grids[f, 5]), int(grids[f, 6])
        sdf.update(g)
        sim.simulate([hair])
        margin = float(np.float32(grids[f, 7]) * np.float32(grids[f, 3]))
        sdf.collide(hair, g, margin)
    for name, buf in (("out_pos", A.BUF_POSITIONS), ("out_prev", A.BUF_POSITIONS_PREV),
                      ("out_prevprev", A.BUF_POSITIONS_PREV_PREV), ("out_tan", A.BUF_TANGENTS),
                      ("out_sld", A.BUF_STRAND_LEVEL_DATA)):
        want = hair.read(buf).view(np.uint32).reshape(-1)
        got = np.frombuffer(d[name], np.uint32)
        assert np.array_equal(got, want), f"{name}: {int((got != want).sum())} words differ"
    cells = int(grids[-1, 4] * grids[-1, 5] * grids[-1, 6])
    assert np.array_equal(np.frombuffer(d["out_sdf"], np.uint32)[:cells], sdf.read(cells))
    # TressFXSDFMarchingCubes on the last grid, at the collision margin, against tfx_mc through Python
    from tressfx_gb300.api import SDFMarchingCubes
    mc = SDFMarchingCubes(ctx, 1 << 17, alloc)
    mc.set_iso_level(float(grids[-1, 7]))
    mc.update(sdf, g)
    want_v, want_n = mc.read()
    assert int(np.frombuffer(d["mc_count"], np.int32)[0]) == want_n and want_n > 100
    assert np.array_equal(np.frombuffer(d["mc_vertices"], np.uint32), want_v.view(np.uint32).reshape(-1))
    mc.close()
    assert (sdf.read(cells).view(np.float32) < 1e10).sum() > 1000
    pos = hair.read(A.BUF_POSITIONS)
    assert np.isfinite(pos).all()
    stamps = d["stamps"].decode().split()
    for want in ("IntegrationAndGlobalShapeContraints", "LocalShapeConstraints", "ConstructSignedDistanceField",
                 "CollideHairVerticesWithSdf"):
        assert want in stamps
    hair.close(); sdf.close(); mesh.close()
