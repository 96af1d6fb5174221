// TressFXSDFMarchingCubes (src/TressFX/TressFXSDFMarchingCubes.cpp:27-233) over the C ABI.
#include "tfx_host_check.h"
#include "tressfx/TressFXSDFMarchingCubes.h"

using tfxhost::check;

TressFXSDFMarchingCubes::TressFXSDFMarchingCubes() : m_MaxMarchingCubesVertices(128 * 1024) {}

TressFXSDFMarchingCubes::TressFXSDFMarchingCubes(int maxVertices) : m_MaxMarchingCubesVertices(maxVertices) {
    if (maxVertices < 0) throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "TressFXSDFMarchingCubes: negative vertex count");
}

TressFXSDFMarchingCubes::~TressFXSDFMarchingCubes() {
    if (m_mc) tfx_mc_destroy(m_mc);
}

void TressFXSDFMarchingCubes::Initialize(const char* /*name*/, EI_Device* pDevice) {
    if (!pDevice) throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "TressFXSDFMarchingCubes::Initialize: null device");
    m_pDevice = pDevice;
}

void TressFXSDFMarchingCubes::Update(EI_CommandContext& commandContext) {
    if (!m_pSDF) throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "TressFXSDFMarchingCubes::Update: no SDF set");
    if (!m_mc) {
        EI_Device* dev = m_pDevice ? m_pDevice : &commandContext.GetDevice();
        check(tfx_mc_create(dev->GetContext(), m_MaxMarchingCubesVertices, m_pSDF->GetGridNumTotalCells(), &m_mc),
              "TressFXSDFMarchingCubes: create");
    }
    check(tfx_mc_set_iso_level(m_mc, m_SDFIsoLevel), "TressFXSDFMarchingCubes: iso level");
    const tfx_sdf_grid g = m_pSDF->GetGrid();
    check(tfx_mc_update(m_mc, m_pSDF->GetHandle(), &g), "TressFXSDFMarchingCubes::Update");
}

EI_Resource TressFXSDFMarchingCubes::GetVerticesGPUBuffer() const {
    void* v = nullptr;
    if (m_mc) check(tfx_mc_get_buffers(m_mc, &v, nullptr), "TressFXSDFMarchingCubes: buffers");
    return EI_Resource(v, (size_t)m_MaxMarchingCubesVertices * 32);
}

int TressFXSDFMarchingCubes::ReadVertices(std::vector<float>& out) const {
    if (!m_mc) throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "TressFXSDFMarchingCubes::ReadVertices: no Update yet");
    out.resize((size_t)m_MaxMarchingCubesVertices * 8);
    int32_t count = 0;
    check(tfx_mc_read(m_mc, out.data(), out.size() * sizeof(float), &count), "TressFXSDFMarchingCubes::ReadVertices");
    return count;
}
