"""The C-ABI library loads without a GPU and exports every function include/tressfx_gb300.h declares."""
import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "tressfx_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b(tfx_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_functions():
    names = declared_functions()
    assert "tfx_hair_create" in names and "tfx_sdf_collide" in names and len(names) > 30


def test_library_exports_every_declared_symbol(built_lib):
    from tressfx_gb300 import _capi
    missing = [n for n in declared_functions() if not hasattr(built_lib, n)]
    assert not missing, f"not exported: {missing}"
    # every declared function is also bound with a prototype in the Python binding
    unbound = [n for n in declared_functions() if n not in _capi.EXPORTED_SYMBOLS]
    assert not unbound, f"declared but not bound in _capi: {unbound}"


def test_dynamic_symbol_table(built_lib):
    from tressfx_gb300 import _capi
    out = subprocess.run(["nm", "-D", "--defined-only", str(_capi.LIB_PATH)], capture_output=True, text=True).stdout
    syms = {line.split()[-1] for line in out.splitlines() if line.strip()}
    for n in declared_functions():
        assert n in syms, n


def test_abi_version_and_status_strings(built_lib):
    assert built_lib.tfx_abi_version() == 1
    assert built_lib.tfx_status_string(0) == b"TFX_OK"
    assert built_lib.tfx_status_string(2) == b"TFX_ERR_VERTS_PER_STRAND"
    assert built_lib.tfx_status_string(999) == b"TFX_ERR_UNKNOWN"


def test_build_targets_sm103a_with_exact_fp_flags():
    from tressfx_gb300 import build as B
    flags = B.nvcc_flags()
    assert "-gencode=arch=compute_103a,code=sm_103a" in flags
    for f in ("-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"):
        assert f in flags


def test_host_library_exports_the_reference_classes(built_lib):
    """libtressfx_host.so carries the C++ host classes with the reference's method names."""
    from tressfx_gb300 import build as B
    assert B.HOST_LIB_PATH.exists()
    out = subprocess.run(["nm", "-DC", "--defined-only", str(B.HOST_LIB_PATH)], capture_output=True, text=True).stdout
    for sym in ("TressFXHairObject::TressFXHairObject(TressFXAsset*, EI_Device*, EI_CommandContext&, char const*, int)",
                "TressFXHairObject::UpdateSimulationParameters(TressFXSimulationSettings const*, float)",
                "TressFXHairObject::UpdateBoneMatrices(AMD::float4x4 const*, int)",
                "TressFXSimulation::Simulate(EI_CommandContext&, std::vector<TressFXHairObject*, std::allocator<TressFXHairObject*> >&)",
                "TressFXSDFCollision::Update(EI_CommandContext&, TressFXSDFCollisionSystem&)",
                "TressFXSDFCollision::CollideWithHair(EI_CommandContext&, TressFXSDFCollisionSystem&, TressFXHairObject&)",
                "TressFXAsset::LoadHairData(_IO_FILE*)", "TressFXAsset::GenerateFollowHairs(int, float, float)",
                "TressFXAsset::ProcessAsset()", "TressFXAsset::LoadBoneData(_IO_FILE*, int, EI_Scene*)",
                "TressFXBoneSkinning::LoadTressFXCollisionMeshData(EI_Scene*, char const*, int, char const*)"):
        assert sym in out, sym
