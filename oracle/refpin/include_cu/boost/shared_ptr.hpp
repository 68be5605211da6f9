// Stand-in for boost::shared_ptr (named only in a typedef of GeometryList.h).
// TEST INFRASTRUCTURE ONLY.
#pragma once
namespace boost {
template <class T>
class shared_ptr {
    T *p;
};
}  // namespace boost
