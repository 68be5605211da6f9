// Stand-in for extensions-CUDA's Convert (used only in log lines of the
// pinned headers).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <Meta/CUDA.h>
namespace OpenEngine {
namespace Utils {
namespace CUDA {
namespace Convert {
template <class T>
inline std::string ToString(const T &) { return std::string(); }
}  // namespace Convert
}  // namespace CUDA
}  // namespace Utils
}  // namespace OpenEngine

// extensions-CUDA's headers bring OpenEngine's namespace into scope; the
// pinned headers rely on it (Utils::CUDA::Convert in IntersectionTests.h).
using namespace OpenEngine;
