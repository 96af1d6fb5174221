"""Row A0, the per-frame constant block, pinned bit for bit to the reference's own code.

oracle/consts_ref compiles TressFXHairObject::UpdateSimulationParameters and SetWind
(src/TressFX/TressFXHairObject.cpp:172-235, 380-437) from the reference tree with the reference's
src/Math.  Three independent producers of the 160-byte TressFXSimulationParams header must agree
word for word: that compiled reference code (here, where the tree is mounted, and through the
committed fixture tests/golden/sim_params_ref.npz everywhere), the oracle's restatement
(tfxo_fill_sim_params) and the library's host code (tfx_fill_sim_params, a host function of the C ABI:
no device is used).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from consts_cases import cases
from tressfx_gb300 import _capi as A
from tressfx_gb300.api import default_settings, fill_sim_params

GOLDEN = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "sim_params_ref.npz")


def oracle_header(st: dict, dt, n, F, frame):
    p = oracle.SimParams()
    it = oracle.fill_sim_params(p, oracle.settings(**st), dt, n, F, frame)
    return p.header_bytes(), it


def library_header(st: dict, dt, n, F, frame):
    s = default_settings()
    for k, v in st.items():
        if k == "wind_direction":
            for i in range(3):
                s.wind_direction[i] = v[i]
        else:
            setattr(s, k, v)
    p = A.SimParams()
    it = fill_sim_params(p, s, dt, n, F, frame)
    return bytes(C.string_at(C.addressof(p), 160)), it


def _words(b: bytes) -> np.ndarray:
    return np.frombuffer(b, dtype=np.uint32)


def _check(name, got, want):
    (gh, gi), (wh, wi) = got, want
    bad = np.nonzero(_words(gh) != _words(wh))[0]
    assert len(bad) == 0 and gi == wi, f"{name}: words {bad.tolist()} differ, CPU iterations {gi} vs {wi}"


def test_fixture_covers_wind_and_iteration_split():
    rows = cases(seed=int(GOLDEN["seed"]), count=int(GOLDEN["count"]))
    assert len(rows) == len(GOLDEN["headers"])
    assert sum(1 for r in rows if r[0]["wind_magnitude"] > 0) > 300
    assert {r[2] for r in rows} == {4, 8, 16, 32, 64}
    assert any(r[4] < 2 for r in rows) and any(r[4] > 10000 for r in rows)


@pytest.mark.parametrize("producer", ["oracle", "library"])
def test_producers_match_the_reference_fixture(built_lib, producer):
    fn = oracle_header if producer == "oracle" else library_header
    rows = cases(seed=int(GOLDEN["seed"]), count=int(GOLDEN["count"]))
    for i, (st, dt, n, F, frame) in enumerate(rows):
        want = (GOLDEN["headers"][i].tobytes(), int(GOLDEN["cpu_iterations"][i]))
        _check(f"{producer} case {i} (n={n}, frame={frame})", fn(st, dt, n, F, frame), want)


def test_producers_match_the_compiled_reference(built_lib):
    R = pytest.importorskip("oracle.consts_ref")
    if R.build() is None:
        pytest.skip("the reference tree is not mounted here")
    for i, (st, dt, n, F, frame) in enumerate(cases(seed=77, count=1500)):
        want = R.update_simulation_parameters(R.settings(**st), dt, n, F, frame)
        _check(f"oracle case {i}", oracle_header(st, dt, n, F, frame), want)
        _check(f"library case {i}", library_header(st, dt, n, F, frame), want)


def test_reference_defaults_match(built_lib):
    R = pytest.importorskip("oracle.consts_ref")
    if R.build() is None:
        pytest.skip("the reference tree is not mounted here")
    ref = R.settings()
    lib = default_settings()
    ora = oracle.settings()
    assert bytes(ref) == bytes(lib) == bytes(ora)
