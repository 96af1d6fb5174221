"""Writes tests/golden/asset_digests.json: per-array SHA-256 digests of what the reference's own
TressFXAsset (compiled by oracle/asset_ref/build.py) produces for the cases of tests/asset_cases.py.

    python tests/golden/make_asset_golden.py
"""
import json
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parent.parent))

from asset_cases import CASES, digests, run_driver  # noqa: E402
from oracle.asset_ref import build as asset_ref  # noqa: E402


def main() -> None:
    exe = asset_ref.build()
    if exe is None:
        raise SystemExit("the reference tree is not available")
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for case in CASES:
            counts, arrays = run_driver(exe, Path(d), case)
            out[case[0]] = digests(counts, arrays)
    (HERE / "asset_digests.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"wrote {len(out)} cases")


if __name__ == "__main__":
    main()
