// TressFXSDFCollision (src/TressFX/TressFXSDFCollision.cpp:38-221) and TressFXBoneSkinning's
// collision-mesh side (src/TressFX/TressFXBoneSkinning.cpp:100-452) over the C ABI.
#include <algorithm>
#include <climits>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "tfx_host_check.h"
#include "tressfx/TressFXBoneSkinning.h"
#include "tressfx/TressFXSDFCollision.h"

using tfxhost::check;

// ============================================================================ TressFXSDFCollision
TressFXSDFCollision::TressFXSDFCollision(EI_Device* pDevice, TressFXSDFInputMeshInterface* pCollMesh,
                                         const char* /*modelName*/, int numCellsInX, float collisionMargin)
    : m_pInputCollisionMesh(pCollMesh), m_CollisionMargin(collisionMargin), m_NumCellsInXAxis(numCellsInX) {
    if (!pDevice || !pCollMesh || numCellsInX <= 0)
        throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "TressFXSDFCollision: null device / mesh or no cells");
    Vector3 bmin, bmax;
    m_pInputCollisionMesh->GetInitialBoundingBox(bmin, bmax);
    const float mn[3] = {bmin.x, bmin.y, bmin.z}, mx[3] = {bmax.x, bmax.y, bmax.z};
    tfx_sdf_grid g;
    float padding = 0.0f;
    int64_t alloc = 0;
    check(tfx_sdf_grid_from_bbox(mn, mx, numCellsInX, &g, &padding, &alloc), "TressFXSDFCollision: grid");
    m_CellSize = g.cell_size;
    m_PaddingBoundary = padding;
    m_Origin = Vector3(g.origin[0], g.origin[1], g.origin[2]);
    m_NumCellsX = g.num_cells_x; m_NumCellsY = g.num_cells_y; m_NumCellsZ = g.num_cells_z;
    m_NumTotalCells = (int)std::min<int64_t>(INT_MAX, alloc);
    Create(pDevice);
}

TressFXSDFCollision::TressFXSDFCollision(EI_Device* pDevice, TressFXSDFInputMeshInterface* pCollMesh,
                                         const char* /*modelName*/, int numCellsX, int numCellsY, int numCellsZ,
                                         float cellSize, float paddingBoundary, float collisionMargin)
    : m_pInputCollisionMesh(pCollMesh), m_CollisionMargin(collisionMargin) {
    if (!pDevice || !pCollMesh || numCellsX <= 0 || numCellsY <= 0 || numCellsZ <= 0 || !(cellSize > 0.0f))
        throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "TressFXSDFCollision: bad explicit grid");
    m_CellSize = cellSize;
    m_PaddingBoundary = paddingBoundary;
    m_NumCellsX = numCellsX; m_NumCellsY = numCellsY; m_NumCellsZ = numCellsZ;
    const int64_t cells = (int64_t)numCellsX * numCellsY * numCellsZ;
    if (cells > INT_MAX) throw TressFXError(TFX_ERR_SIZE, "TressFXSDFCollision: grid too large");
    m_NumTotalCells = (int)cells;
    Vector3 bmin, bmax;
    m_pInputCollisionMesh->GetInitialBoundingBox(bmin, bmax);
    UpdateSDFGrid(bmin, bmax);
    Create(pDevice);
}

void TressFXSDFCollision::Create(EI_Device* pDevice) {
    check(tfx_sdf_create(pDevice->GetContext(), m_NumTotalCells, &m_sdf), "TressFXSDFCollision: grid buffer");
    void* p = nullptr;
    size_t bytes = 0;
    check(tfx_sdf_get_buffer(m_sdf, &p, &bytes), "TressFXSDFCollision: grid buffer");
    m_SignedDistanceField = EI_Resource(p, bytes);
    BindMesh();
}

void TressFXSDFCollision::BindMesh() {
    check(tfx_sdf_set_mesh(m_sdf, m_pInputCollisionMesh->GetMeshBuffer().GetDevicePointer(),
                           m_pInputCollisionMesh->GetNumMeshVertices(),
                           static_cast<const uint32_t*>(m_pInputCollisionMesh->GetTrimeshVertexIndicesBuffer().GetDevicePointer()),
                           m_pInputCollisionMesh->GetNumMeshTriangle()),
          "TressFXSDFCollision: mesh");
}

TressFXSDFCollision::~TressFXSDFCollision() {
    if (m_sdf) tfx_sdf_destroy(m_sdf);
}

// UpdateSDFGrid (TressFXSDFCollision.cpp:88-93): origin = tight bbox min - padding.
void TressFXSDFCollision::UpdateSDFGrid(const Vector3& tightBBoxMin, const Vector3& /*tightBBoxMax*/) {
    const float mn[3] = {tightBBoxMin.x, tightBBoxMin.y, tightBBoxMin.z};
    tfx_sdf_grid g = GetGrid();
    check(tfx_sdf_grid_origin(mn, m_PaddingBoundary.x, &g), "UpdateSDFGrid");
    m_Origin = Vector3(g.origin[0], g.origin[1], g.origin[2]);
}

tfx_sdf_grid TressFXSDFCollision::GetGrid() const {
    tfx_sdf_grid g;
    std::memset(&g, 0, sizeof(g));
    g.origin[0] = m_Origin.x; g.origin[1] = m_Origin.y; g.origin[2] = m_Origin.z; g.origin[3] = 0.0f;
    g.cell_size = m_CellSize;
    g.num_cells_x = m_NumCellsX; g.num_cells_y = m_NumCellsY; g.num_cells_z = m_NumCellsZ;
    return g;
}

void TressFXSDFCollision::Update(EI_CommandContext& commandContext, TressFXSDFCollisionSystem& system) {
    if (!m_pInputCollisionMesh) return;
    Vector3 mn, mx;
    m_pInputCollisionMesh->GetBoundingBox(mn, mx);
    UpdateSDFGrid(mn, mx);
    BindMesh();   // the mesh interface may hand out new buffers
    EI_Device& device = system.GetDevice() ? *system.GetDevice() : commandContext.GetDevice();
    const tfx_sdf_grid g = GetGrid();
    check(tfx_sdf_dispatch(m_sdf, TFX_KERNEL_SDF_INITIALIZE, &g), "InitializeSignedDistanceField");
    device.GetTimeStamp("InitializeSignedDistanceField");
    check(tfx_sdf_dispatch(m_sdf, TFX_KERNEL_SDF_CONSTRUCT, &g), "ConstructSignedDistanceField");
    device.GetTimeStamp("ConstructSignedDistanceField");
    check(tfx_sdf_dispatch(m_sdf, TFX_KERNEL_SDF_FINALIZE, &g), "FinalizeSignedDistanceField");
    device.GetTimeStamp("FinalizeSignedDistanceField");
}

void TressFXSDFCollision::CollideWithHair(EI_CommandContext& commandContext, TressFXSDFCollisionSystem& system,
                                          TressFXHairObject& hairObject) {
    if (!m_pInputCollisionMesh) return;
    EI_Device& device = system.GetDevice() ? *system.GetDevice() : commandContext.GetDevice();
    const tfx_sdf_grid g = GetGrid();
    check(tfx_sdf_collide(m_sdf, hairObject.GetHandle(), &g, m_CollisionMargin * m_CellSize), "CollideHairVerticesWithSdf");
    device.GetTimeStamp("CollideHairVerticesWithSdf");
}

// ============================================================================ TressFXBoneSkinning
TressFXBoneSkinning::~TressFXBoneSkinning() {
    if (m_mesh) tfx_mesh_destroy(m_mesh);
}

bool TressFXBoneSkinning::LoadTressFXCollisionMeshData(EI_Scene* scene, const char* filePath, int skinNumber,
                                                       const char* followBone) {
    if (!scene || !filePath) return false;
    std::ifstream stream(filePath);
    if (!stream.is_open()) return false;
    auto tokens_of = [](const std::string& line) {
        std::vector<std::string> t;
        std::istringstream is(line);
        std::string s;
        while (is >> s) t.push_back(s);
        return t;
    };
    // the next line that is neither empty nor a comment
    auto next_data_line = [&](std::vector<std::string>& t) {
        std::string line;
        while (std::getline(stream, line)) {
            if (line.empty() || line[0] == '#') continue;
            t = tokens_of(line);
            if (!t.empty()) return true;
        }
        return false;
    };
    std::vector<std::string> boneNames;
    std::vector<float> vertices, skinning;
    std::vector<uint32_t> indices;
    int numVertices = 0, numTriangles = 0;
    std::string line;
    while (std::getline(stream, line)) {
        if (line.empty() || line[0] == '#') continue;
        const std::vector<std::string> t = tokens_of(line);
        if (t.empty()) continue;
        const std::string& token = t[0];
        if (token.find("numOfBones") != std::string::npos) {
            if (t.size() < 2) return false;
            const int numOfBones = std::atoi(t[1].c_str());
            for (int b = 0; b < numOfBones; ++b) {
                std::vector<std::string> bt;
                if (!next_data_line(bt) || bt.size() < 2) return false;
                boneNames.push_back(bt[1]);
            }
        }
        if (token.find("numOfVertices") != std::string::npos) {
            if (t.size() < 2) return false;
            numVertices = std::atoi(t[1].c_str());
            if (numVertices <= 0) return false;
            vertices.assign((size_t)numVertices * 8, 0.0f);
            skinning.assign((size_t)numVertices * 8, 0.0f);
            for (int v = 0; v < numVertices; ++v) {
                std::vector<std::string> vt;
                if (!next_data_line(vt) || vt.size() != 15 || std::atoi(vt[0].c_str()) != v) return false;
                for (int k = 0; k < 3; ++k) {
                    vertices[8 * v + k] = (float)std::atof(vt[1 + k].c_str());
                    vertices[8 * v + 4 + k] = (float)std::atof(vt[4 + k].c_str());
                }
                for (int k = 0; k < 4; ++k) {
                    const int bi = std::atoi(vt[7 + k].c_str());
                    if (bi < 0 || bi >= (int)boneNames.size()) return false;
                    skinning[8 * v + k] = (float)scene->GetBoneIdByName(skinNumber, boneNames[bi].c_str());
                    skinning[8 * v + 4 + k] = (float)std::atof(vt[11 + k].c_str());
                }
            }
        } else if (token.find("numOfTriangles") != std::string::npos) {
            if (t.size() < 2) return false;
            numTriangles = std::atoi(t[1].c_str());
            if (numTriangles <= 0) return false;
            indices.assign((size_t)numTriangles * 3, 0);
            for (int tr = 0; tr < numTriangles; ++tr) {
                std::vector<std::string> tt;
                if (!next_data_line(tt) || tt.size() != 4 || std::atoi(tt[0].c_str()) != tr) return false;
                for (int k = 0; k < 3; ++k) indices[3 * tr + k] = (uint32_t)std::atoi(tt[1 + k].c_str());
            }
        }
    }
    if (numVertices <= 0 || numTriangles <= 0) return false;
    m_vertices.swap(vertices);
    m_skinning.swap(skinning);
    m_tempIndices.swap(indices);
    m_NumVertices = numVertices;
    m_NumTriangles = numTriangles;
    m_followBone = scene->GetBoneIdByName(skinNumber, followBone ? followBone : "");
    return true;
}

void TressFXBoneSkinning::SetMeshData(const float* vertices, int numVertices, const uint32_t* indices, int numTriangles,
                                      const float* boneSkinning, int followBone) {
    if (!vertices || !indices || !boneSkinning || numVertices <= 0 || numTriangles <= 0)
        throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "TressFXBoneSkinning::SetMeshData: bad argument");
    m_vertices.assign(vertices, vertices + (size_t)numVertices * 8);
    m_tempIndices.assign(indices, indices + (size_t)numTriangles * 3);
    m_skinning.assign(boneSkinning, boneSkinning + (size_t)numVertices * 8);
    m_NumVertices = numVertices;
    m_NumTriangles = numTriangles;
    m_followBone = followBone;
}

void TressFXBoneSkinning::Initialize(EI_Device* pDevice, EI_CommandContext& /*commandContext*/, const char* /*name*/) {
    if (!pDevice || m_NumVertices <= 0) throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "TressFXBoneSkinning: no mesh loaded");
    if (m_mesh) { tfx_mesh_destroy(m_mesh); m_mesh = nullptr; }
    check(tfx_mesh_create(pDevice->GetContext(), m_vertices.data(), m_NumVertices, m_tempIndices.data(), m_NumTriangles,
                          m_skinning.data(), &m_mesh),
          "TressFXBoneSkinning");
    void* sk = nullptr;
    void* ix = nullptr;
    int32_t nv = 0, nt = 0;
    check(tfx_mesh_get_buffers(m_mesh, &sk, &ix, &nv, &nt), "TressFXBoneSkinning");
    m_skinned = EI_Resource(sk, (size_t)nv * 32);
    m_indices = EI_Resource(ix, (size_t)nt * 12);

    // bounding sphere of the bind pose as a cube (TressFXBoneSkinning.cpp:388-399)
    Vector3 center(0.0f, 0.0f, 0.0f);
    for (int i = 0; i < m_NumVertices; ++i) center = center + Vector3(m_vertices[8 * i], m_vertices[8 * i + 1], m_vertices[8 * i + 2]);
    const float cnt = (float)m_NumVertices;
    center = Vector3(center.x / cnt, center.y / cnt, center.z / cnt);
    float radius = 0.0f;
    for (int i = 0; i < m_NumVertices; ++i) {
        const Vector3 d = Vector3(m_vertices[8 * i], m_vertices[8 * i + 1], m_vertices[8 * i + 2]) - center;
        radius = fmaxf(radius, d.Length());
    }
    m_bbMin = Vector3(center.x - radius, center.y - radius, center.z - radius);
    m_bbMax = Vector3(center.x + radius, center.y + radius, center.z + radius);
}

void TressFXBoneSkinning::Update(EI_CommandContext& /*commandContext*/, const AMD::float4x4* boneMatrices, int numBones) {
    if (!m_mesh) throw TressFXError(TFX_ERR_INVALID_ARGUMENT, "TressFXBoneSkinning::Update before Initialize");
    check(tfx_mesh_skin(m_mesh, boneMatrices ? boneMatrices[0].m : nullptr, numBones), "TressFXBoneSkinning::Update");
    if (boneMatrices && m_followBone >= 0 && m_followBone < numBones) m_followMatrix = boneMatrices[m_followBone];
}

// GetBoundingBox (TressFXBoneSkinning.cpp:439-452): the initial box moved with its centre by the
// follow bone, centre' = [centre 1] * M.
void TressFXBoneSkinning::GetBoundingBox(Vector3& min, Vector3& max) {
    const float* M = m_followMatrix.m;
    const Vector3 c((m_bbMax.x + m_bbMin.x) / 2.0f, (m_bbMax.y + m_bbMin.y) / 2.0f, (m_bbMax.z + m_bbMin.z) / 2.0f);
    float nc[3];
    for (int k = 0; k < 3; ++k) nc[k] = ((c.x * M[0 * 4 + k] + c.y * M[1 * 4 + k]) + c.z * M[2 * 4 + k]) + 1.0f * M[3 * 4 + k];
    const Vector3 d(nc[0] - c.x, nc[1] - c.y, nc[2] - c.z);
    min = m_bbMin + d;
    max = m_bbMax + d;
}
