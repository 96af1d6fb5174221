"""Writes tests/golden/asset_digests.json: per-array SHA-256 digests of what the reference's own
TressFXAsset (compiled by oracle/asset_ref/build.py) produces for the cases of tests/asset_cases.py and
for its shipped Ratboy mohawk, and of what its own .tfxmesh parser (oracle/mesh_ref) reads from the
shipped Ratboy collision meshes.

    python tests/golden/make_asset_golden.py
"""
import json
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parent.parent))

from asset_cases import CASES, REAL_ASSET_DIR, REAL_HAIR, REAL_MESHES, digests, mesh_digests, run_driver, \
    run_mesh_driver, run_real_hair  # noqa: E402
from oracle.asset_ref import build as asset_ref  # noqa: E402
import oracle.mesh_ref as mesh_ref  # noqa: E402


def main() -> None:
    exe = asset_ref.build()
    if exe is None:
        raise SystemExit("the reference tree is not available")
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for case in CASES:
            counts, arrays = run_driver(exe, Path(d), case)
            out[case[0]] = digests(counts, arrays)
        # the reference's shipped Ratboy asset through its own loaders
        counts, arrays = run_real_hair(exe, Path(d))
        out[REAL_HAIR[0]] = digests(counts, arrays)
        mexe = mesh_ref.build()
        for m in REAL_MESHES:
            counts, arrays = run_mesh_driver(mexe, Path(d), REAL_ASSET_DIR / m)
            out[m] = mesh_digests(counts, arrays)
    (HERE / "asset_digests.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"wrote {len(out)} cases")


if __name__ == "__main__":
    main()
