// TressFXSDFInputMeshInterface (src/TressFX/TressFXSDFInputMeshInterface.h:33-57): what an SDF
// needs from its collision mesh.  The mesh buffer is DEVICE memory of {float4 position, float4
// normal}[GetNumMeshVertices()], the index buffer DEVICE uint32[3 * GetNumMeshTriangle()].
#pragma once

#include "EngineInterface.h"
#include "TressFXCommon.h"

class TressFXSDFInputMeshInterface {
public:
    virtual ~TressFXSDFInputMeshInterface() {}
    virtual EI_Resource& GetMeshBuffer() = 0;
    virtual EI_Resource& GetTrimeshVertexIndicesBuffer() = 0;
    virtual int GetNumMeshVertices() = 0;
    virtual int GetNumMeshTriangle() = 0;
    virtual size_t GetSizeOfMeshElement() = 0;
    virtual void GetBoundingBox(Vector3& min, Vector3& max) = 0;
    virtual void GetInitialBoundingBox(Vector3& min, Vector3& max) = 0;
};
