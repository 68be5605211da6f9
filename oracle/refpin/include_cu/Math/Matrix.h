// Stand-in for OpenEngine's Math::Matrix (a member type of GeometryList,
// never used by the traversal).  TEST INFRASTRUCTURE ONLY.
#pragma once
namespace OpenEngine {
namespace Math {
template <unsigned int M, unsigned int N, class T>
class Matrix {
    T e[M * N];
};
}  // namespace Math
}  // namespace OpenEngine
