"""Writes tests/golden/sim_params_ref.npz from the reference's own constant code.

Run where the reference checkout is mounted:  python tests/golden/make_consts_golden.py
oracle/consts_ref compiles TressFXHairObject::UpdateSimulationParameters and SetWind
(src/TressFX/TressFXHairObject.cpp:172-235, 380-437) as they stand in the reference tree.  This
script draws seeded settings, strand shapes and frames (tests/consts_cases.py), runs them through
that code, and stores the 160-byte constant-block headers and CPU local-iteration counts, so that
the pin travels to machines without the reference tree.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from consts_cases import cases  # noqa: E402


def main() -> None:
    import oracle.consts_ref as R
    if R.build() is None:
        raise SystemExit("the reference sources are not mounted here")
    rows = cases(seed=2024, count=600)
    headers = np.zeros((len(rows), 160), dtype=np.uint8)
    iters = np.zeros(len(rows), dtype=np.int32)
    for i, (st, dt, n, F, frame) in enumerate(rows):
        h, it = R.update_simulation_parameters(R.settings(**st), dt, n, F, frame)
        headers[i] = np.frombuffer(h, dtype=np.uint8)
        iters[i] = it
    out = ROOT / "tests" / "golden" / "sim_params_ref.npz"
    np.savez_compressed(out, seed=np.int32(2024), count=np.int32(len(rows)), headers=headers, cpu_iterations=iters)
    print(out, out.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
