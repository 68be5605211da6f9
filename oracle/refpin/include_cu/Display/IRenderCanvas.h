// Stand-in for OpenEngine's IRenderCanvas (used only by the tracers' host
// Trace methods, which the pin test never calls).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <Math/Matrix.h>
namespace OpenEngine {
namespace Display {
class IViewingVolume;
class IRenderCanvas {
public:
    virtual ~IRenderCanvas() {}
    virtual unsigned int GetWidth() const = 0;
    virtual unsigned int GetHeight() const = 0;
    virtual IViewingVolume *GetViewingVolume() = 0;
};
}  // namespace Display
}  // namespace OpenEngine
