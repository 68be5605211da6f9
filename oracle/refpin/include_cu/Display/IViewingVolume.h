// Stand-in for OpenEngine's IViewingVolume (declared only).  TEST
// INFRASTRUCTURE ONLY.
#pragma once
#include <Math/Matrix.h>
namespace OpenEngine {
namespace Display {
class IViewingVolume {
public:
    virtual ~IViewingVolume() {}
};
}  // namespace Display
}  // namespace OpenEngine
