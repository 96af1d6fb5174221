// TressFXSDFCollisionSystem / TressFXSDFCollision (src/TressFX/TressFXSDFCollision.h:39-118): a
// signed distance grid rebuilt from a collision mesh and collided with hair, sized and placed by the
// reference's rules (TressFXSDFCollision.cpp:38-93).
#pragma once

#include "EngineInterface.h"
#include "TressFXHairObject.h"
#include "TressFXSDFInputMeshInterface.h"

class TressFXSDFCollisionSystem {
public:
    // The reference creates its four compute PSOs here; the kernels are linked in, so this only
    // records the device.
    void Initialize(EI_Device* pDevice) { m_device = pDevice; }
    EI_Device* GetDevice() const { return m_device; }
private:
    EI_Device* m_device = nullptr;
};

class TressFXSDFCollision : private TressFXNonCopyable {
public:
    TressFXSDFCollision(EI_Device* pDevice, TressFXSDFInputMeshInterface* pCollMesh, const char* modelName,
                        int numCellsInX, float collisionMargin);
    // Explicit grid: dimensions, cell size and padding given instead of derived from numCellsInX
    // (a grid such as 64^3 with a 2 cm margin cannot come out of the reference's sizing rule).
    TressFXSDFCollision(EI_Device* pDevice, TressFXSDFInputMeshInterface* pCollMesh, const char* modelName,
                        int numCellsX, int numCellsY, int numCellsZ, float cellSize, float paddingBoundary,
                        float collisionMargin);
    ~TressFXSDFCollision();

    // Rebuilds the grid around the mesh's current bounding box (Initialize, Construct, Finalize).
    void Update(EI_CommandContext& commandContext, TressFXSDFCollisionSystem& system);
    // CollideHairVerticesWithSdf_forward on every vertex of the hair object.
    void CollideWithHair(EI_CommandContext& commandContext, TressFXSDFCollisionSystem& system,
                         TressFXHairObject& hairObject);

    float GetSDFCollisionMargin() const { return m_CollisionMargin; }
    EI_Resource& GetSDFDataGPUBuffer() { return m_SignedDistanceField; }
    const EI_Resource& GetSDFDataGPUBuffer() const { return m_SignedDistanceField; }
    float GetGridCellSize() const { return m_CellSize; }
    Vector3 GetGridOrigin() const { return m_Origin; }
    void GetGridNumCells(int& x, int& y, int& z) const { x = m_NumCellsX; y = m_NumCellsY; z = m_NumCellsZ; }
    int GetGridNumTotalCells() const { return m_NumTotalCells; }

    tfx_sdf GetHandle() const { return m_sdf; }
    // This frame's grid as the C ABI describes it.
    tfx_sdf_grid GetGrid() const;

private:
    void Create(EI_Device* pDevice);
    void UpdateSDFGrid(const Vector3& tightBBoxMin, const Vector3& tightBBoxMax);
    void BindMesh();

    TressFXSDFInputMeshInterface* m_pInputCollisionMesh = nullptr;
    float m_CollisionMargin = 0.0f;
    int m_NumCellsInXAxis = 0;
    float m_GridAllocationMutliplier = 1.4f;
    float m_CellSize = 0.0f;
    Vector3 m_PaddingBoundary;
    Vector3 m_Origin;
    int m_NumCellsX = 0, m_NumCellsY = 0, m_NumCellsZ = 0;
    int m_NumTotalCells = 0;
    tfx_sdf m_sdf = nullptr;
    EI_Resource m_SignedDistanceField;
};
