// Stand-in for OpenEngine's ISceneNodeVisitor (GeometryList's base class).
// TEST INFRASTRUCTURE ONLY.
#pragma once
namespace OpenEngine {
namespace Scene {
class RenderStateNode;
class OscCUDAMeshNode;
class ISceneNodeVisitor {
public:
    virtual ~ISceneNodeVisitor() {}
};
}  // namespace Scene
}  // namespace OpenEngine
