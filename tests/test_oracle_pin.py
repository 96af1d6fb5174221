"""Pins the oracle to the reference's own compute shaders compiled as C++ (oracle/hlsl_ref).

Runs only where the reference checkout is mounted (the translation reads its HLSL files); the
golden fixtures carry the same check everywhere else.  Every kernel is compared after every
dispatch, bit for bit, over scenes that exercise each strand length, follow hairs, wind, reset
frames, skinning and the SDF build / collide path.
"""
import numpy as np
import pytest

from oracle import hlsl_ref

pytestmark = pytest.mark.skipif(not hlsl_ref.available(), reason="reference shader sources not mounted")

KEYS = ("pos", "prev", "prevprev", "tan", "sld")


def scenes():
    from tressfx_gb300 import synthetic as S
    out = []
    for n in (4, 8, 16, 32, 64):
        sc = S.scene_small(seed=300 + n, num_guides=64 if n > 4 else 128, n=n)
        sc.objects[0].settings.update(local_constraints_iterations=2, length_constraints_iterations=2,
                                      wind_magnitude=2.0, global_constraint_stiffness=0.3, global_constraints_range=0.6)
        out.append((f"n{n}", sc))
    out.append(("head", S.scene_head(seed=9, num_guides=128, n=16, follows=3, triangles=2500, sdf_cells=28, frames=5)))
    return out


@pytest.mark.parametrize("name,scene", scenes(), ids=lambda x: x if isinstance(x, str) else "")
def test_oracle_equals_reference_every_kernel(oracle_lib, name, scene):
    from oracle.scene_driver import OraclePipeline
    from tressfx_gb300.headless import FrameInputs
    import oracle
    ref = hlsl_ref.RefPipeline(scene)
    ora = OraclePipeline(scene)
    for f in range(5):
        fin = FrameInputs(scene, f)
        # oracle side, stage by stage, in lock-step with the reference
        for i, c in enumerate(ora.consts):
            c.update_simulation_parameters(fin.settings_overrides[i], scene.dt)
            c.update_bone_matrices(fin.hair_bones[i])
        mismatches = []

        def check(k, r):
            h = ora.hair[0]
            c = ora.consts[0]
            for _ in range(c.cpu_local_iterations if k == 4 else 1):
                h.stage(k, c.current_params())
            for key in KEYS:
                if not np.array_equal(getattr(h, key).view(np.uint32), getattr(r.hair[0], key).view(np.uint32)):
                    mismatches.append((f, k, key))

        o = scene.objects[0]
        if o.mesh is not None:
            skinned = oracle.mesh_skin(o.mesh.vertices, o.mesh.skinning, fin.mesh_bones[0])
            ora.sdf_words[0] = oracle.sdf_build(fin.grids[0], skinned, o.mesh.indices)
        ref.step(fin, per_stage=check)
        for c in ora.consts:
            c.increase_simulation_frame()
        if o.mesh is not None:
            assert np.array_equal(ref.skinned[0], skinned), f"frame {f}: mesh skinning"
            assert np.array_equal(ref.sdf_words[0], ora.sdf_words[0]), f"frame {f}: SDF"
            g = fin.grids[0]
            oracle.sdf_collide(g, ora.sdf_words[0], ora._margin_world(o, g), ora.hair[0])
            for key in KEYS:
                assert np.array_equal(getattr(ora.hair[0], key), getattr(ref.hair[0], key)), f"frame {f} collide {key}"
        assert not mismatches, mismatches
